// Surface patches, quadrature and local forms; CSR pattern; segmented scatter.
//
// One warp assembles one cut tet (grid-stride over the active tets):
//   patch   lanes 0..7 take the 8 sub-tets of the order-2 principal lattice
//           (PrincipalLatticeCL, geom/principallattice.cpp:33-79), classify
//           their sign pattern through the 81-entry facet table
//           (RefPatchBuilderCL<3>::assign, geom/reftetracut.cpp:53-60) and
//           place their facets with a warp scan -- facet order is the
//           reference's (sub-tet order, table order);
//   points  lanes take the 7 Quad5_2D nodes of the facets (num/discretize.cpp:
//           263-294, weights |det| (x1/2 on lattice faces), num/quadrature.tpp:
//           265-314), 32 points per round, and stage weight, basis values and
//           surface gradients (I - n n^T) grad(phi) in shared memory, with
//           n = grad(phi_h)/|grad(phi_h)| of the P2 level set
//           (LocalAssembler::buildNormal, surfactant/ifacetransp.h:1066-1072);
//   forms   lanes own entries (i <= j) of the symmetric element matrices and
//           sum over the staged points (quad_2D, num/quadrature.tpp:31-108);
//           C_n uses the 15-point Quad5 rule on the tet times |det J|.
// Element matrices go to a packed buffer; the CSR values are then formed by a
// segmented sum over contributions sorted by (row, column, tet), i.e. in the
// reference's triangulation-order accumulation, without atomics.
#include <climits>

#include <cub/device/device_radix_sort.cuh>

#include "ff.cuh"
#include "tf_internal.cuh"

namespace tf {

// ---------------------------------------------------------------------------
// constant tables (built on the host at first use)
// ---------------------------------------------------------------------------
struct Tables {
    double lat_v[10][4];    // lattice vertices (barycentric)
    int lat_t[8][4];        // lattice sub-tets
    int can_a[8][6];        // cut-edge orientation of the first sub-tet holding the edge
    int can_b[8][6];
    int ledge[8][6];        // lattice edge id 0..24
    int edge_a[25], edge_b[25];  // canonical endpoints of every lattice edge
    int reg_child[8][4];         // regular children in P2-DoF numbering (ChildDataAr, geom/topo.cpp:333-341)
    signed char pat_nf[81]; // facets per sign pattern (-1: all-zero pattern)
    signed char pat_bnd[81];
    signed char pat_f[81][2][3];  // ext ids: 0..3 vertex, 4..9 edge + 4
    double q2_node[7][3], q2_w[7];
    double q3_node[15][4], q3_w[15], q3_sw[15];  // q3_sw = sqrt(q3_w)
    double qq2_node[4][3], qq2_w[4];  // Quad2_2D (legacy numbering)
    int sym_i[55], sym_j[55];  // packed upper triangle, NL = 10
    int sym4_i[10], sym4_j[10];  // NL = 4
};
__constant__ Tables cT;
static bool g_tables_ready[64] = {false};

__constant__ int cP2OnLat[10] = {0, 4, 7, 9, 1, 2, 5, 3, 6, 8};  // p2_dof_on_lattice_2

static void build_tables(Tables& T) {
    // lattice of order 2 (PrincipalLatticeCL ctor and create_tetras)
    const int n = 2;
    int nv = 0;
    for (int x = 0; x <= n; ++x)
        for (int y = 0; y <= x; ++y)
            for (int z = 0; z <= y; ++z, ++nv) {
                T.lat_v[nv][0] = (double)(n - x) / n;
                T.lat_v[nv][1] = (double)(x - y) / n;
                T.lat_v[nv][2] = (double)(y - z) / n;
                T.lat_v[nv][3] = (double)z / n;
            }
    auto vidx = [](int i, int j, int k) {
        return (i > 0 ? ((i + 2) * (i + 1) * i) / 6 : 0) + (j > 0 ? ((j + 1) * j) / 2 : 0) + k;
    };
    static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    int nt = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j)
            for (int k = 0; k <= j; ++k)
                for (int l = 0; l < 6; ++l) {
                    int t[4][3] = {{i, j, k}};
                    bool ok = true;
                    for (int s = 1; s < 4 && ok; ++s) {
                        for (int q = 0; q < 3; ++q) t[s][q] = t[s - 1][q];
                        ++t[s][perm[l][s - 1]];
                        ok = n >= t[s][0] && t[s][0] >= t[s][1] && t[s][1] >= t[s][2];
                    }
                    if (!ok) continue;
                    for (int s = 0; s < 4; ++s) T.lat_t[nt][s] = vidx(t[s][0], t[s][1], t[s][2]);
                    ++nt;
                }
    // canonical cut-edge orientation and lattice edge ids
    int seen_a[64], seen_b[64], nseen = 0;
    for (int s = 0; s < 8; ++s)
        for (int e = 0; e < 6; ++e) {
            const int a = T.lat_t[s][ev0(e)], b = T.lat_t[s][ev1(e)];
            const int lo = a < b ? a : b, hi = a < b ? b : a;
            int id = -1;
            for (int q = 0; q < nseen; ++q)
                if ((seen_a[q] < seen_b[q] ? seen_a[q] : seen_b[q]) == lo &&
                    (seen_a[q] < seen_b[q] ? seen_b[q] : seen_a[q]) == hi)
                    id = q;
            if (id < 0) {
                id = nseen++;
                seen_a[id] = a;
                seen_b[id] = b;
            }
            T.can_a[s][e] = seen_a[id];
            T.can_b[s][e] = seen_b[id];
            T.ledge[s][e] = id;
        }
    for (int q = 0; q < 25; ++q) {
        T.edge_a[q] = seen_a[q];
        T.edge_b[q] = seen_b[q];
    }
    static const int reg[8][4] = {{0, 4, 5, 7}, {4, 1, 6, 8}, {4, 5, 6, 8}, {4, 5, 7, 8},
                                  {5, 6, 2, 9}, {5, 6, 8, 9}, {5, 7, 8, 9}, {7, 8, 9, 3}};
    for (int c = 0; c < 8; ++c)
        for (int k = 0; k < 4; ++k) T.reg_child[c][k] = reg[c][k];
    // sign-pattern facet table (SignTraitsCL<3>::compute_cuts + RefPatchBuilderCL<3>::assign)
    for (int p = 0; p < 81; ++p) {
        int sg[4], q = p, sum = 0;
        for (int k = 0; k < 4; ++k) {
            sg[k] = (q % 3) - 1;
            q /= 3;
            sum += sg[k];
        }
        // index = sum (s_k + 1) 3^k
        T.pat_nf[p] = 0;
        T.pat_bnd[p] = 0;
        if (sg[0] == 0 && sg[1] == 0 && sg[2] == 0 && sg[3] == 0) {
            T.pat_nf[p] = -1;
            continue;
        }
        int cut[4], nr = 0, nrv = 0;
        if (sum != 4 && sum != -4) {
            for (int k = 0; k < 4; ++k)
                if (sg[k] == 0) cut[nrv++] = k;
            nr = nrv;
            for (int e = 0; e < 6; ++e)
                if (sg[ev0(e)] * sg[ev1(e)] == -1) cut[nr++] = e + 4;
        }
        if (nr < 3) continue;
        T.pat_nf[p] = (signed char)(nr - 2);
        T.pat_bnd[p] = nrv == 3;
        for (int f = 0; f + 2 < nr; ++f)
            for (int j = 0; j < 3; ++j) T.pat_f[p][f][j] = (signed char)cut[f + j];
    }
    // quadrature rules (Quad5_2DDataCL, Quad5DataCL, Quad2_2DDataCL)
    const double s15 = std::sqrt(15.0);
    const double A1 = (6.0 - s15) / 21.0, B1 = (9.0 + 2.0 * s15) / 21.0;
    const double A2 = (6.0 + s15) / 21.0, B2 = (9.0 - 2.0 * s15) / 21.0;
    const double n2[7][3] = {{1. / 3., 1. / 3., 1. / 3.}, {A1, A1, B1}, {A1, B1, A1}, {B1, A1, A1},
                             {A2, A2, B2}, {A2, B2, A2}, {B2, A2, A2}};
    for (int i = 0; i < 7; ++i)
        for (int j = 0; j < 3; ++j) T.q2_node[i][j] = n2[i][j];
    T.q2_w[0] = 9. / 80.;
    for (int i = 1; i <= 3; ++i) T.q2_w[i] = (155. - s15) / 2400.;
    for (int i = 4; i <= 6; ++i) T.q2_w[i] = (155. + s15) / 2400.;
    const double a1 = (7.0 - s15) / 34.0, b1 = (13.0 + 3.0 * s15) / 34.0;
    const double a2 = (7.0 + s15) / 34.0, b2 = (13.0 - 3.0 * s15) / 34.0;
    const double a3 = (10.0 - 2.0 * s15) / 40.0, b3 = (10.0 + 2.0 * s15) / 40.0;
    const double n3[15][4] = {{0.25, 0.25, 0.25, 0.25}, {a1, a1, a1, b1}, {a1, a1, b1, a1}, {a1, b1, a1, a1},
                              {b1, a1, a1, a1},         {a2, a2, a2, b2}, {a2, a2, b2, a2}, {a2, b2, a2, a2},
                              {b2, a2, a2, a2},         {a3, a3, b3, b3}, {a3, b3, a3, b3}, {a3, b3, b3, a3},
                              {b3, a3, a3, b3},         {b3, a3, b3, a3}, {b3, b3, a3, a3}};
    for (int i = 0; i < 15; ++i)
        for (int j = 0; j < 4; ++j) T.q3_node[i][j] = n3[i][j];
    T.q3_w[0] = 0.01975308641975308641975308641975308641975;
    for (int i = 1; i <= 4; ++i) T.q3_w[i] = 0.01198951396316977000173064248499538621936;
    for (int i = 5; i <= 8; ++i) T.q3_w[i] = 0.01151136787104539754677023934921978132914;
    for (int i = 9; i <= 14; ++i) T.q3_w[i] = 0.008818342151675485008818342151675485008818;
    for (int i = 0; i < 15; ++i) T.q3_sw[i] = std::sqrt(T.q3_w[i]);
    const double qq[4][3] = {{1., 0., 0.}, {0., 1., 0.}, {0., 0., 1.}, {1. / 3., 1. / 3., 1. / 3.}};
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 3; ++j) T.qq2_node[i][j] = qq[i][j];
    T.qq2_w[0] = T.qq2_w[1] = T.qq2_w[2] = 1. / 24.;
    T.qq2_w[3] = 0.375;
    int k = 0;
    for (int i = 0; i < 10; ++i)
        for (int j = i; j < 10; ++j, ++k) {
            T.sym_i[k] = i;
            T.sym_j[k] = j;
        }
    k = 0;
    for (int i = 0; i < 4; ++i)
        for (int j = i; j < 4; ++j, ++k) {
            T.sym4_i[k] = i;
            T.sym4_j[k] = j;
        }
}

int ensure_tables(Context* c) {
    if (c->device >= 0 && c->device < 64 && g_tables_ready[c->device]) return TF_OK;
    Tables T;
    build_tables(T);
    TF_CUDA(c, cudaMemcpyToSymbol(cT, &T, sizeof(Tables)));
    if (c->device >= 0 && c->device < 64) g_tables_ready[c->device] = true;
    return TF_OK;
}

// ---------------------------------------------------------------------------
// per-tet geometry shared by the kernels
// ---------------------------------------------------------------------------
struct TetGeom {
    double X[4][3];   // vertex coordinates
    double gl[4][3];  // world gradients of the barycentric coordinates (T * ref grads)
    double G[4][3];   // gradient of the P2 level set at the 4 vertices (linear field)
    double absdet;    // |det J|
};

// GetTrafoTr (geom/multigrid.h:603-623), P1 gradients and the vertex values
// of grad(phi_h) for the P2 level set ls10 (4 vertex + 6 edge values).
// Tet geometry (GetTrafoTr, geom/multigrid.h:627-650) on the warp.  Lanes
// 0..8 form the edge matrix M (M[r][c] = X[c+1][r] - X[0][r]) and its
// cofactors, the warp takes one reciprocal of det M, and lanes 0..11 form the
// barycentric gradients gl (T = cof(M) / det) and the gradient coefficients G
// of the P2 level set.  On GB300 an FP64 instruction costs the same with one
// active lane as with 32, so spreading the work over lanes divides its cost.
__device__ inline void warp_tet_geometry(TetGeom& g, const double* ls10, double* Ms, double* Cs, int lane) {
    if (lane < 9) {
        const int r = lane / 3, c = lane % 3;
        Ms[lane] = g.X[c + 1][r] - g.X[0][r];
    }
    __syncwarp();
    if (lane < 9) {
        const int r = lane / 3, c = lane % 3;
        const int r1 = (r + 1) % 3, r2 = (r + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
        Cs[lane] = Ms[3 * r1 + c1] * Ms[3 * r2 + c2] - Ms[3 * r1 + c2] * Ms[3 * r2 + c1];
    }
    __syncwarp();
    const double d = Ms[0] * Cs[0] + Ms[1] * Cs[1] + Ms[2] * Cs[2];
    const double inv = 1.0 / d;
    if (lane < 12) {
        const int v = lane / 3, r = lane % 3;
        g.gl[v][r] = v == 0 ? (-(Cs[3 * r] * inv) - Cs[3 * r + 1] * inv) - Cs[3 * r + 2] * inv : Cs[3 * r + v - 1] * inv;
    }
    if (lane == 0) g.absdet = fabs(d);
    __syncwarp();
    // grad H_i(e_v) = (4 delta_iv - 1) gl_i ; grad H_ab(e_v) = 4 (delta_bv gl_a + delta_av gl_b)
    if (lane < 12) {
        const int v = lane / 3, r = lane % 3;
        double s = 0.;
        for (int i = 0; i < 4; ++i) s += ls10[i] * ((i == v ? 3. : -1.) * g.gl[i][r]);
        for (int e = 0; e < 6; ++e) {
            const int a = ev0(e), b = ev1(e);
            if (b == v) s += ls10[4 + e] * (4. * g.gl[a][r]);
            if (a == v) s += ls10[4 + e] * (4. * g.gl[b][r]);
        }
        g.G[v][r] = s;
    }
    __syncwarp();
}

// 1/sqrt(s) to FP64 accuracy: FP32 seed and two Newton steps
// y <- y (3/2 - s/2 y^2) (relative error ~1e-16); FP64 division and square
// root are long instruction sequences on the FP64 pipe, this is ~10 operations.
__device__ inline double rsqrt_fp64(double s) {
    if (!(s > 1e-30 && s < 1e30)) return 1.0 / sqrt(s);
    double y = (double)rsqrtf((float)s);
    const double h = 0.5 * s;
    y = y * (1.5 - h * y * y);
    y = y * (1.5 - h * y * y);
    return y;
}

__device__ inline void unit_normal(const TetGeom& g, const double b[4], double n[3]) {
    double v[3];
    for (int r = 0; r < 3; ++r) v[r] = b[0] * g.G[0][r] + b[1] * g.G[1][r] + b[2] * g.G[2][r] + b[3] * g.G[3][r];
    const double inv = rsqrt_fp64(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    n[0] = v[0] * inv;
    n[1] = v[1] * inv;
    n[2] = v[2] * inv;
}

// Surface gradients scale (I - n n^T) grad(phi_i) and values phi_i at
// barycentric b (the scale, sqrt of the point weight, enters through the four
// projected grad(lambda_v), which every surface gradient combines linearly).
// grad(phi_i) = sum_v c_iv(b) grad(lambda_v) with at most two terms (P2:
// vertex i: (4 b_i - 1) grad(lambda_i); edge (a,c): 4 b_c grad(lambda_a) +
// 4 b_a grad(lambda_c)), so the projection is applied to the four
// grad(lambda_v) once and combined afterwards.
template <bool P2>
__device__ inline void surf_basis(const TetGeom& g, const double b[4], const double n[3], double scale, double* phi,
                                  double (*sg)[3]) {
    double pg[4][3];
    for (int v = 0; v < 4; ++v) {
        const double ng = n[0] * g.gl[v][0] + n[1] * g.gl[v][1] + n[2] * g.gl[v][2];
        for (int r = 0; r < 3; ++r) pg[v][r] = scale * (g.gl[v][r] - ng * n[r]);
    }
    if constexpr (!P2) {
        for (int i = 0; i < 4; ++i) {
            phi[i] = b[i];
            for (int r = 0; r < 3; ++r) sg[i][r] = pg[i][r];
        }
    } else {
        double q[4];
        for (int i = 0; i < 4; ++i) {
            q[i] = 4. * b[i];
            phi[i] = b[i] * (2. * b[i] - 1.);
            const double f = q[i] - 1.;
            for (int r = 0; r < 3; ++r) sg[i][r] = f * pg[i][r];
        }
        for (int e = 0; e < 6; ++e) {
            const int a = ev0(e), c = ev1(e);
            phi[4 + e] = q[a] * b[c];
            for (int r = 0; r < 3; ++r) sg[4 + e][r] = q[c] * pg[a][r] + q[a] * pg[c][r];
        }
    }
}

// scale n . grad(phi_i) at barycentric b (volume stabilisation; the scale,
// sqrt of the point weight, enters through the four n . grad(lambda_v))
template <bool P2>
__device__ inline void normal_derivs(const TetGeom& g, const double b[4], const double n[3], double scale,
                                     double* dn) {
    double ng[4];
    for (int v = 0; v < 4; ++v) ng[v] = scale * (n[0] * g.gl[v][0] + n[1] * g.gl[v][1] + n[2] * g.gl[v][2]);
    if constexpr (!P2) {
        for (int i = 0; i < 4; ++i) dn[i] = ng[i];
    } else {
        for (int i = 0; i < 4; ++i) dn[i] = (4. * b[i] - 1.) * ng[i];
        for (int e = 0; e < 6; ++e) {
            const int a = ev0(e), c = ev1(e);
            dn[4 + e] = 4. * (b[c] * ng[a] + b[a] * ng[c]);
        }
    }
}

template <bool P2>
__device__ inline void basis(const TetGeom& g, const double b[4], double* phi, double (*grad)[3]) {
    if constexpr (!P2) {
        for (int i = 0; i < 4; ++i) {
            phi[i] = b[i];
            for (int r = 0; r < 3; ++r) grad[i][r] = g.gl[i][r];
        }
    } else {
        for (int i = 0; i < 4; ++i) {
            phi[i] = b[i] * (2. * b[i] - 1.);
            const double f = 4. * b[i] - 1.;
            for (int r = 0; r < 3; ++r) grad[i][r] = f * g.gl[i][r];
        }
        for (int e = 0; e < 6; ++e) {
            const int a = ev0(e), c = ev1(e);
            phi[4 + e] = 4. * b[a] * b[c];
            for (int r = 0; r < 3; ++r) grad[4 + e][r] = 4. * (b[c] * g.gl[a][r] + b[a] * g.gl[c][r]);
        }
    }
}

struct RhsPar {
    int kind;
    double p[8];
};
__device__ inline double rhs_value(const RhsPar& R, const double x[3]) {
    if (R.kind == TF_RHS_CONST) return R.p[0];
    if (R.kind == TF_RHS_SPHERE_XYZ) {
        const double d0 = x[0] - R.p[0], d1 = x[1] - R.p[1], d2 = x[2] - R.p[2];
        const double n2 = d0 * d0 + d1 * d1 + d2 * d2;
        const double inv = rsqrt_fp64(n2);
        const double dist = n2 * inv - R.p[3];
        const double s = dist * inv;
        const double y0 = x[0] - s * d0, y1 = x[1] - s * d1, y2 = x[2] - s * d2;
        return R.p[4] * y0 * y1 * y2;
    }
    return 0.;
}

__device__ inline void set_status(int* st, int code, int64_t where) {
    if (atomicCAS(st, 0, code) == 0) st[1] = (int)where;
}


__device__ inline void sym_entry(int nl, int k, int& i, int& j) {
    if (nl == 10) {
        i = cT.sym_i[k];
        j = cT.sym_j[k];
    } else {
        i = cT.sym4_i[k];
        j = cT.sym4_j[k];
    }
}
__host__ __device__ inline int sym_index(int nl, int i, int j) {
    if (i > j) {
        const int t = i;
        i = j;
        j = t;
    }
    return i * nl - (i * (i - 1)) / 2 + (j - i);
}

// ---------------------------------------------------------------------------
// the warp's patch: facets of the 8 lattice sub-tets (sub-tet order)
// ---------------------------------------------------------------------------
struct PatchSmem {
    double fb[16][3][4];  // facet vertices, barycentric
    double fw[16];        // |det| of the facet, x1/2 on lattice faces
    int bnd[16];
    int nf;
    double cut[25][4];    // cut point of each lattice edge (where the edge is cut)
    int fsub[16], floc[16], fpat[16];  // owning sub-tet, facet index in its pattern, pattern
};

// cut point of a lattice edge: ConvexComb(ls_a/(ls_a - ls_b), v_a, v_b)
// (MergeCutPolicyCL::operator(), geom/subtriangulation.h:514-524), rounded
// like the reference (no contraction).
__device__ inline void cut_point(const double* lat, int a, int b, double out[4]) {
    const double t = __ddiv_rn(lat[a], __dsub_rn(lat[a], lat[b]));
    const double s = __dsub_rn(1.0, t);
    for (int c = 0; c < 4; ++c) out[c] = __dadd_rn(__dmul_rn(s, cT.lat_v[a][c]), __dmul_rn(t, cT.lat_v[b][c]));
}

// All lanes call.  Lanes 0..24 compute the cut point of one lattice edge each
// (every edge once, with its canonical orientation, so all sub-tets sharing
// an edge see the same point, as MergeCutPolicyCL's memo gives); lanes 0..7
// classify one sub-tet each and list its facets; then one lane per facet
// forms the facet's vertices and |det|.  Returns the facet count.
__device__ int warp_patch(const double ls10[10], const double X[4][3], PatchSmem& P, int lane, int* status,
                          int64_t tet) {
    double lat[10];
    for (int k = 0; k < 10; ++k) lat[cP2OnLat[k]] = ls10[k];
    if (lane < 25) {
        const int a = cT.edge_a[lane], b = cT.edge_b[lane];
        const double va = lat[a], vb = lat[b];
        if ((va > 0. && vb < 0.) || (va < 0. && vb > 0.)) {
            double cp[4];
            cut_point(lat, a, b, cp);
            for (int c = 0; c < 4; ++c) P.cut[lane][c] = cp[c];
        }
    }
    int nf = 0, pat = 0;
    if (lane < 8) {
        for (int k = 0; k < 4; ++k) {
            const double v = lat[cT.lat_t[lane][k]];
            pat += ((v > 0.) - (v < 0.) + 1) * (k == 0 ? 1 : k == 1 ? 3 : k == 2 ? 9 : 27);
        }
        nf = cT.pat_nf[pat];
        if (nf < 0) {
            set_status(status, TF_ERR_ZERO_PATTERN, tet);
            nf = 0;
        }
    }
    int incl = nf;
    for (int o = 1; o < 8; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 7);
    if (lane < 8)
        for (int f = 0; f < nf; ++f) {
            const int k = incl - nf + f;
            P.fsub[k] = lane;
            P.floc[k] = f;
            P.fpat[k] = pat;
        }
    __syncwarp();
    if (lane < total) {
        const int sub = P.fsub[lane], f = P.floc[lane], fp = P.fpat[lane];
        double w[3][3];
        for (int j = 0; j < 3; ++j) {
            const int ext = cT.pat_f[fp][f][j];
            double b[4];
            if (ext < 4) {
                const int L = cT.lat_t[sub][ext];
                for (int c = 0; c < 4; ++c) b[c] = cT.lat_v[L][c];
            } else {
                const int id = cT.ledge[sub][ext - 4];
                for (int c = 0; c < 4; ++c) b[c] = P.cut[id][c];
            }
            for (int c = 0; c < 4; ++c) P.fb[lane][j][c] = b[c];
            for (int r = 0; r < 3; ++r) w[j][r] = X[0][r] * b[0] + X[1][r] * b[1] + X[2][r] * b[2] + X[3][r] * b[3];
        }
        double u[3], v[3];
        for (int r = 0; r < 3; ++r) {
            u[r] = w[1][r] - w[0][r];
            v[r] = w[2][r] - w[0][r];
        }
        const double c0 = u[1] * v[2] - u[2] * v[1], c1 = u[2] * v[0] - u[0] * v[2], c2 = u[0] * v[1] - u[1] * v[0];
        const int bnd = cT.pat_bnd[fp];
        P.fw[lane] = sqrt(c0 * c0 + c1 * c1 + c2 * c2) * (bnd ? 0.5 : 1.0);
        P.bnd[lane] = bnd;
    }
    if (lane == 0) P.nf = total;
    __syncwarp();
    return total;
}

// ---------------------------------------------------------------------------
// assembly kernel: warp per active tet
// ---------------------------------------------------------------------------
constexpr int kAsmWarps = 4;

template <int NL>
struct AsmSmem {
    TetGeom g;
    double gM[9], gC[9];  // edge matrix and cofactors
    double ls10[10];
    PatchSmem P;
    double w[32];
    double phi[32][NL];   // also n.grad(phi) for the volume rule
    double sg[32][NL][3];
    double mob[32];
    double fx[32];  // sqrt(w) f(x_p): the load vector is sum_p (sqrt(w) f)(sqrt(w) phi_i)
    double wind[NL == 4 ? 30 : 1];    // N_P1P1: P2 wind at the 10 nodes, xyz
    double wn[NL == 4 ? 32 : 1][4];   // sqrt(w) (wind . surface gradient of phi_j)
    // linear level set on the tet (P1 forms): constant surface gradients of
    // the hat functions, their Gram matrix (packed) and n . grad(phi_i)
    double lin_sg[NL == 4 ? 4 : 1][3];
    double lin_G[NL == 4 ? 10 : 1];
    double lin_dn[NL == 4 ? 4 : 1];
};

struct AsmArgs {
    MeshView M;
    const double* lsv;
    const double* lse;
    int64_t n_active;
    const int32_t* active;
    const int32_t* l2g;
    unsigned forms;
    RhsPar rhs;
    const double* chi;  // P1 DOF vector for LaplaceM (NULL: mobility 1)
    int degenerate;
    double* elem;       // [form][n_active][nsym]
    double* elem_rhs;   // [n_active][NL]
    int* status;
    const double* windv;  // N_P1P1 wind, xyz per vertex / edge
    const double* winde;
    double* elem_n;       // [n_active][16]: N_P1P1, row i col j
    // pair forms: the per-tet records of active tets [c0, c1) (k_prep_tets)
    void* prep;
    int64_t c0, c1;
    const int32_t* prep_order;  // prep thread i takes active tet c0 + prep_order[i] (null: c0 + i)
};

template <int NL>
__global__ void __launch_bounds__(32 * kAsmWarps) k_assemble(AsmArgs A) {
    constexpr bool P2 = NL == 10;
    constexpr int NSYM = NL * (NL + 1) / 2;
    constexpr int EPL = (NSYM + 31) / 32;  // entries per lane
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    AsmSmem<NL>& S = reinterpret_cast<AsmSmem<NL>*>(smem_raw)[wib];
    const bool wantM = A.forms & (1u << TF_FORM_M), wantA = A.forms & (1u << TF_FORM_A);
    const bool wantC = A.forms & (1u << TF_FORM_CN), wantL = A.forms & (1u << TF_FORM_LAPM);
    const bool wantF = A.rhs.kind != TF_RHS_NONE;
    const bool wantN = NL == 4 && (A.forms & (1u << TF_FORM_N));
    const int64_t nwarps = (int64_t)gridDim.x * kAsmWarps;

    for (int64_t r = (int64_t)blockIdx.x * kAsmWarps + wib; r < A.n_active; r += nwarps) {
        const int32_t t = A.active[r];
        int32_t v[4], e[6];
        mesh_tet(A.M, t, v, e);
        if (lane < 4) {
            double x[3];
            mesh_coord(A.M, v[lane], x);
            for (int c = 0; c < 3; ++c) S.g.X[lane][c] = x[c];
            S.ls10[lane] = A.lsv[v[lane]];
        } else if (lane < 10) {
            S.ls10[lane] = A.lse[e[lane - 4]];
        }
        if constexpr (NL == 4) {
            if (wantN && lane < 30) {  // node k = lane / 3: vertices 0..3, edges 4..9
                const int k = lane / 3, r = lane - 3 * (lane / 3);
                S.wind[lane] = k < 4 ? A.windv[3 * (int64_t)v[k] + r] : A.winde[3 * (int64_t)e[k - 4] + r];
            }
        }
        __syncwarp();
        warp_tet_geometry(S.g, S.ls10, S.gM, S.gC, lane);
        double ls10[10];
        for (int k = 0; k < 10; ++k) ls10[k] = S.ls10[k];
        __syncwarp();
        const int nf = warp_patch(ls10, S.g.X, S.P, lane, A.status, t);
        // A P1 level set is stored as a P2 vector whose edge values are the
        // means of the end values.  Where that holds bit for bit on all six
        // edges, the level set is linear on the tet: grad(phi_h) and the normal
        // are constant, and so are the surface gradients sg_i of the P1 hat
        // functions.  Then A_ij = (sum_p w_p) sg_i.sg_j, LaplaceM_ij =
        // (sum_p w_p mob_p) sg_i.sg_j and C_ij = |det| (sum_q w_q) dn_i dn_j:
        // the same integrals as the per-point evaluation (which differs only by
        // rounding), without the per-point normals and projections that make
        // up most of the FP64 work.  (warp-uniform)
        bool lin = false;
        if constexpr (NL == 4) {
            lin = true;
            for (int k = 0; k < 6; ++k) {
                const double mean = __dmul_rn(0.5, __dadd_rn(ls10[ev0(k)], ls10[ev1(k)]));
                lin = lin && __double_as_longlong(mean) == __double_as_longlong(ls10[4 + k]);
            }
            if (lin) {
                const double bc[4] = {0.25, 0.25, 0.25, 0.25};
                double n[3];
                unit_normal(S.g, bc, n);
                if (lane < 12) {
                    const int v = lane / 3, c = lane - 3 * (lane / 3);
                    const double ng = n[0] * S.g.gl[v][0] + n[1] * S.g.gl[v][1] + n[2] * S.g.gl[v][2];
                    S.lin_sg[v][c] = S.g.gl[v][c] - ng * n[c];
                }
                __syncwarp();
                if (lane < 10) {
                    int i, j;
                    sym_entry(4, lane, i, j);
                    S.lin_G[lane] = S.lin_sg[j][0] * S.lin_sg[i][0] + S.lin_sg[j][1] * S.lin_sg[i][1] +
                                    S.lin_sg[j][2] * S.lin_sg[i][2];
                } else if (lane < 14) {
                    const int i = lane - 10;
                    S.lin_dn[i] = n[0] * S.g.gl[i][0] + n[1] * S.g.gl[i][1] + n[2] * S.g.gl[i][2];
                }
                __syncwarp();
            }
        }
        double chi_loc[4] = {0, 0, 0, 0};
        if (wantL && A.chi && A.degenerate)
            for (int k = 0; k < 4; ++k) chi_loc[k] = A.chi[A.l2g[r * NL + k]];

        double accM[EPL], accA[EPL], accL[EPL], accC[EPL];
        for (int q = 0; q < EPL; ++q) accM[q] = accA[q] = accL[q] = accC[q] = 0.;
        double accF = 0., accN = 0.;
        const int npts = 7 * nf;
        for (int base = 0; base < npts; base += 32) {
            const int p = base + lane;
            if (p < npts) {
                const int f = p / 7, q = p - 7 * (p / 7);
                double b[4];
                for (int c = 0; c < 4; ++c)
                    b[c] = S.P.fb[f][0][c] * cT.q2_node[q][0] + S.P.fb[f][1][c] * cT.q2_node[q][1] +
                           S.P.fb[f][2][c] * cT.q2_node[q][2];
                const double w = S.P.fw[f] * cT.q2_w[q];
                // values are stored times sqrt(w): sum_p w u_i u_j = sum_p (sqrt(w) u_i)(sqrt(w) u_j)
                const double sw = w > 0. ? w * rsqrt_fp64(w) : 0.;
                double phi[NL], sg[NL][3];  // sg: surface gradients times sqrt(w)
                if (NL == 4 && lin) {
                    for (int i = 0; i < NL; ++i) phi[i] = b[i];
                } else {
                    double n[3];
                    unit_normal(S.g, b, n);
                    surf_basis<P2>(S.g, b, n, sw, phi, sg);
                }
                S.w[lane] = sw;
                for (int i = 0; i < NL; ++i) {
                    S.phi[lane][i] = sw * phi[i];
                    if (!(NL == 4 && lin))
                        for (int c = 0; c < 3; ++c) S.sg[lane][i][c] = sg[i][c];
                }
                if (wantL) {
                    double m = 1.0;
                    if (A.chi && A.degenerate) {
                        const double ch = chi_loc[0] * b[0] + chi_loc[1] * b[1] + chi_loc[2] * b[2] + chi_loc[3] * b[3];
                        m = ch * (1. - ch);
                        if (m < 0.) m = 0.;
                    }
                    S.mob[lane] = m;
                }
                if (wantF) {
                    double x[3];
                    for (int c = 0; c < 3; ++c)
                        x[c] = S.g.X[0][c] * b[0] + S.g.X[1][c] * b[1] + S.g.X[2][c] * b[2] + S.g.X[3][c] * b[3];
                    S.fx[lane] = sw * rhs_value(A.rhs, x);
                }
                if constexpr (NL == 4) {
                    // N_P1P1: the P2 wind at the point (LocalP2CL at b: vertex
                    // b_i (2 b_i - 1), edge (a,c) 4 b_a b_c) dotted with the
                    // surface gradients of the hat functions
                    if (wantN) {
                        double h[10];
                        for (int i = 0; i < 4; ++i) h[i] = b[i] * (2. * b[i] - 1.);
                        for (int k = 0; k < 6; ++k) h[4 + k] = 4. * b[ev0(k)] * b[ev1(k)];
                        double wv[3] = {0., 0., 0.};
                        for (int k = 0; k < 10; ++k)
                            for (int c = 0; c < 3; ++c) wv[c] += S.wind[3 * k + c] * h[k];
                        for (int j = 0; j < 4; ++j) {
                            if (lin) {
                                const double* g = S.lin_sg[j];
                                S.wn[lane][j] = sw * (wv[0] * g[0] + wv[1] * g[1] + wv[2] * g[2]);
                            } else {  // sg carries sqrt(w) already
                                S.wn[lane][j] = wv[0] * sg[j][0] + wv[1] * sg[j][1] + wv[2] * sg[j][2];
                            }
                        }
                    }
                }
            }
            __syncwarp();
            const int cnt = min(32, npts - base);
            // P1: 10 entries x 3 point groups on 30 lanes, F: 4 rows x 8 groups
            // (groups combined after the last chunk); P2: 55 entries on 2 x 32 lanes
            constexpr int kGroups = NL == 4 ? 3 : 1;
            const int grp = NL == 4 ? lane / 10 : 0;
            for (int q = 0; q < EPL; ++q) {
                const int k = NL == 4 ? lane % 10 : lane + 32 * q;
                if (k >= NSYM || grp >= kGroups) break;
                int i, j;
                sym_entry(NL, k, i, j);
                double sm = accM[q], sa = accA[q], sl = accL[q];
                for (int pp = grp; pp < cnt; pp += kGroups) {
                    if (wantM) sm += S.phi[pp][j] * S.phi[pp][i];
                    if (wantA || wantL) {
                        // linear level set: the point weight (times sg_i.sg_j after the sum)
                        const double d = (NL == 4 && lin)
                                             ? S.w[pp] * S.w[pp]
                                             : S.sg[pp][j][0] * S.sg[pp][i][0] + S.sg[pp][j][1] * S.sg[pp][i][1] +
                                                   S.sg[pp][j][2] * S.sg[pp][i][2];
                        sa += d;
                        if (wantL) sl += S.mob[pp] * d;
                    }
                }
                accM[q] = sm;
                accA[q] = sa;
                accL[q] = sl;
            }
            if constexpr (NL == 4) {
                if (wantF)
                    for (int pp = lane >> 2; pp < cnt; pp += 8) accF += S.fx[pp] * S.phi[pp][lane & 3];
                // N: 16 entries (i, j) = (lane / 4 % 4, lane % 4) on 2 point groups
                if (wantN) {
                    const int i = (lane >> 2) & 3, j = lane & 3;
                    for (int pp = lane >> 4; pp < cnt; pp += 2) accN += S.phi[pp][i] * S.wn[pp][j];
                }
            } else if (wantF && lane < 30) {
                // P2: 10 rows x 3 point groups (combined after the last chunk)
                const int i = lane % 10;
                for (int pp = lane / 10; pp < cnt; pp += 3) accF += S.fx[pp] * S.phi[pp][i];
            }
            __syncwarp();
        }
        if constexpr (NL == 4) {
            // combine the point groups in a fixed order: entries (g0 + g1) + g2, F tree over 8 groups
            const double m1 = __shfl_down_sync(0xffffffffu, accM[0], 10), m2 = __shfl_down_sync(0xffffffffu, accM[0], 20);
            const double a1 = __shfl_down_sync(0xffffffffu, accA[0], 10), a2 = __shfl_down_sync(0xffffffffu, accA[0], 20);
            const double l1 = __shfl_down_sync(0xffffffffu, accL[0], 10), l2 = __shfl_down_sync(0xffffffffu, accL[0], 20);
            accM[0] = (accM[0] + m1) + m2;
            accA[0] = (accA[0] + a1) + a2;
            accL[0] = (accL[0] + l1) + l2;
            if (lin && lane < 10) {  // sum_p w_p (and w_p mob_p) times the constant sg_i.sg_j
                accA[0] *= S.lin_G[lane];
                accL[0] *= S.lin_G[lane];
            }
            accF += __shfl_down_sync(0xffffffffu, accF, 16);
            accF += __shfl_down_sync(0xffffffffu, accF, 8);
            accF += __shfl_down_sync(0xffffffffu, accF, 4);
            accN += __shfl_down_sync(0xffffffffu, accN, 16);  // point groups: g0 + g1
        } else if (wantF) {
            // P2 load vector: point groups (g0 + g1) + g2
            const double f1 = __shfl_down_sync(0xffffffffu, accF, 10), f2 = __shfl_down_sync(0xffffffffu, accF, 20);
            accF = (accF + f1) + f2;
        }
        if (NL == 4 && wantC && lin) {
            // constant n . grad(phi_i): the 15-point rule reduces to its weight sum
            double s3 = 0.;
            for (int pp = 0; pp < 15; ++pp) s3 += cT.q3_w[pp];
            int i, j;
            sym_entry(4, lane % 10, i, j);
            accC[0] = (s3 * (S.lin_dn[j] * S.lin_dn[i])) * S.g.absdet;
        } else if (wantC) {
            // normal-gradient volume stabilisation on the 15-point Quad5 rule
            if (lane < 15) {
                double b[4];
                for (int c = 0; c < 4; ++c) b[c] = cT.q3_node[lane][c];
                double n[3];
                unit_normal(S.g, b, n);
                double dn[NL];
                normal_derivs<P2>(S.g, b, n, cT.q3_sw[lane], dn);
                for (int i = 0; i < NL; ++i) S.phi[lane][i] = dn[i];
            }
            __syncwarp();
            if constexpr (NL == 4) {
                double sc = 0.;
                if (lane < 30) {
                    int i, j;
                    sym_entry(NL, lane % 10, i, j);
                    for (int pp = lane / 10; pp < 15; pp += 3) sc += S.phi[pp][j] * S.phi[pp][i];
                }
                const double s1 = __shfl_down_sync(0xffffffffu, sc, 10), s2 = __shfl_down_sync(0xffffffffu, sc, 20);
                accC[0] = ((sc + s1) + s2) * S.g.absdet;
            } else {
                for (int q = 0; q < EPL; ++q) {
                    const int k = lane + 32 * q;
                    if (k >= NSYM) break;
                    int i, j;
                    sym_entry(NL, k, i, j);
                    double sc = 0.;
                    for (int pp = 0; pp < 15; ++pp) sc += S.phi[pp][j] * S.phi[pp][i];
                    accC[q] = sc * S.g.absdet;
                }
            }
            __syncwarp();
        }
        // write the packed element matrices
        for (int q = 0; q < EPL; ++q) {
            const int k = lane + 32 * q;
            if (k >= NSYM) break;
            if (wantM) A.elem[((int64_t)TF_FORM_M * A.n_active + r) * NSYM + k] = accM[q];
            if (wantA) A.elem[((int64_t)TF_FORM_A * A.n_active + r) * NSYM + k] = accA[q];
            if (wantC) A.elem[((int64_t)TF_FORM_CN * A.n_active + r) * NSYM + k] = accC[q];
            if (wantL) A.elem[((int64_t)TF_FORM_LAPM * A.n_active + r) * NSYM + k] = accL[q];
        }
        if (wantF && lane < NL) A.elem_rhs[r * NL + lane] = accF;
        if (wantN && lane < 16) A.elem_n[r * 16 + lane] = accN;
        __syncwarp();
    }
}

#include "asm_pair.cuh"

// The order of the prep threads over active tets [A.c0, A.c1): by the sign
// pattern of each tet's lattice values (k_prep_key), so that a warp's tets
// take the same branches.  Every thread still writes its own tet's record.
static int prep_order(Context* c, AsmArgs& A, int64_t chunk) {
    A.prep_order = nullptr;
    if (!c->prep_sort) return TF_OK;
    const int64_t n = A.c1 - A.c0;
    TF_TRY(ensure(c, c->prep_key, (size_t)(2 * chunk)));
    TF_TRY(ensure(c, c->prep_idx, (size_t)(2 * chunk)));
    uint32_t* key = c->prep_key.p;
    int32_t* idx = c->prep_idx.p;
    k_prep_key<<<grid_for(c, n, 256), 256, 0, c->stream>>>(A, key, idx);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    size_t bytes = 0;
    TF_CUDA(c, cub::DeviceRadixSort::SortPairs(nullptr, bytes, key, key + chunk, idx, idx + chunk, (int)n, 0,
                                                kPrepKeyBits, c->stream));
    TF_TRY(ensure(c, c->prep_tmp, bytes + 1));
    TF_CUDA(c, cub::DeviceRadixSort::SortPairs(c->prep_tmp.p, bytes, key, key + chunk, idx, idx + chunk, (int)n, 0,
                                                kPrepKeyBits, c->stream));
    A.prep_order = idx + chunk;
    return TF_OK;
}

// ---------------------------------------------------------------------------
// CSR pattern: contributions bucketed by row, sorted by (column, contribution)
// ---------------------------------------------------------------------------
constexpr int kRowCap = 1024;  // contributions per row handled by one warp

// Contributions of the active tets to every row.  Entries of unnumbered DOFs
// (-1, legacy numbering) and tets with mask[r] == 0 are left out, as the
// reference's MatrixBuilderCL only receives numbered pairs of visited tets.
__global__ void k_row_counts(int64_t n_active, int nl, const int32_t* __restrict__ l2g, const uint8_t* __restrict__ mask,
                             int32_t* __restrict__ cnt) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n_active * nl;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = q / nl;
        const int32_t row = l2g[q];
        if (row < 0 || (mask && !mask[r])) continue;
        int nc = 0;
        for (int j = 0; j < nl; ++j) nc += l2g[r * nl + j] >= 0;
        atomicAdd(&cnt[row], nc);
    }
}

__global__ void k_bucket(int64_t n_active, int nl, const int32_t* __restrict__ l2g, const uint8_t* __restrict__ mask,
                         const int32_t* __restrict__ start, int32_t* __restrict__ cursor, uint64_t* __restrict__ contrib) {
    const int nl2 = nl * nl;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n_active * nl2;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = c / nl2;
        const int ij = (int)(c - r * nl2);
        const int i = ij / nl, j = ij - (ij / nl) * nl;
        const int32_t row = l2g[r * nl + i], col = l2g[r * nl + j];
        if (row < 0 || col < 0 || (mask && !mask[r])) continue;
        const int32_t pos = start[row] + atomicAdd(&cursor[row], 1);
        contrib[pos] = ((uint64_t)(uint32_t)col << 32) | (uint64_t)(uint32_t)c;
    }
}

// warp per row: bitonic sort of the row's keys in shared memory, unique count
__global__ void k_row_sort(int64_t m, const int32_t* __restrict__ start, uint64_t* __restrict__ contrib,
                           int32_t* __restrict__ ucnt, int* __restrict__ status) {
    __shared__ uint64_t buf[4][kRowCap];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint64_t* b = buf[wib];
    for (int64_t row = (int64_t)blockIdx.x * 4 + wib; row < m; row += (int64_t)gridDim.x * 4) {
        const int32_t s = start[row], n = start[row + 1] - start[row];
        if (n > kRowCap) {
            if (lane == 0) set_status(status, TF_ERR_CAPACITY, row);
            continue;
        }
        int np = 1;
        while (np < n) np <<= 1;
        for (int k = lane; k < np; k += 32) b[k] = k < n ? contrib[s + k] : ~0ull;
        __syncwarp();
        for (int size = 2; size <= np; size <<= 1)
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int k = lane; k < np; k += 32) {
                    const int partner = k ^ stride;
                    if (partner > k) {
                        const bool up = (k & size) == 0;
                        const uint64_t a = b[k], c = b[partner];
                        if ((a > c) == up) {
                            b[k] = c;
                            b[partner] = a;
                        }
                    }
                }
                __syncwarp();
            }
        int u = 0;
        for (int k = lane; k < n; k += 32) {
            contrib[s + k] = b[k];
            u += (k == 0) || ((b[k] >> 32) != (b[k - 1] >> 32));
        }
        for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(0xffffffffu, u, o);
        if (lane == 0) ucnt[row] = u;
        __syncwarp();
    }
}

// warp per row: column indices, segment starts, diagonal slot
__global__ void k_row_emit(int64_t m, const int32_t* __restrict__ start, const uint64_t* __restrict__ contrib,
                           const int32_t* __restrict__ rowptr, int32_t* __restrict__ colind,
                           int32_t* __restrict__ seg_start, int32_t* __restrict__ diag_slot) {
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int64_t row = (int64_t)blockIdx.x * 4 + wib; row < m; row += (int64_t)gridDim.x * 4) {
        const int32_t s = start[row], n = start[row + 1] - start[row];
        int32_t carry = rowptr[row];
        for (int k0 = 0; k0 < n; k0 += 32) {
            const int k = k0 + lane;
            int head = 0;
            uint32_t col = 0;
            if (k < n) {
                col = (uint32_t)(contrib[s + k] >> 32);
                head = (k == 0) || (col != (uint32_t)(contrib[s + k - 1] >> 32));
            }
            const unsigned mask = __ballot_sync(0xffffffffu, head);
            if (head) {
                const int32_t slot = carry + __popc(mask & ((1u << lane) - 1));
                colind[slot] = (int32_t)col;
                seg_start[slot] = s + k;
                if ((int64_t)col == row) diag_slot[row] = slot;
            }
            carry += __popc(mask);
        }
    }
}

// segmented sums: vals[f][slot] = sum over the slot's contributions (tet order)
template <int NL>
__global__ void k_scatter(int64_t nnz, const int32_t* __restrict__ seg_start, const uint64_t* __restrict__ contrib,
                          int64_t n_active, const double* __restrict__ elem, unsigned forms, double* v0, double* v1,
                          double* v2, double* v3, const double* __restrict__ elem_n = nullptr, double* v4 = nullptr) {
    constexpr int NSYM = NL * (NL + 1) / 2;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t s = seg_start[k], e = seg_start[k + 1];
        double a0 = 0., a1 = 0., a2 = 0., a3 = 0., a4 = 0.;
        for (int32_t p = s; p < e; ++p) {
            const uint32_t c = (uint32_t)contrib[p];
            const uint32_t r = c / (NL * NL);
            const int ij = (int)(c - r * (NL * NL));
            const int64_t idx = (int64_t)r * NSYM + sym_index(NL, ij / NL, ij % NL);
            if (forms & 1u) a0 += elem[idx];
            if (forms & 2u) a1 += elem[(int64_t)TF_FORM_A * n_active * NSYM + idx];
            if (forms & 4u) a2 += elem[(int64_t)TF_FORM_CN * n_active * NSYM + idx];
            if (forms & 8u) a3 += elem[(int64_t)TF_FORM_LAPM * n_active * NSYM + idx];
            // N (not symmetric): row-local i = ij / NL, column-local j = ij % NL
            if (NL == 4 && (forms & (1u << TF_FORM_N))) a4 += elem_n[(int64_t)r * 16 + ij];
        }
        if (forms & 1u) v0[k] = a0;
        if (forms & 2u) v1[k] = a1;
        if (forms & 4u) v2[k] = a2;
        if (forms & 8u) v3[k] = a3;
        if (NL == 4 && (forms & (1u << TF_FORM_N))) v4[k] = a4;
    }
}

// load vector: the diagonal slot of a row lists exactly its (tet, i) pairs
template <int NL>
__global__ void k_scatter_rhs(int64_t m, const int32_t* __restrict__ diag_slot, const int32_t* __restrict__ seg_start,
                              const uint64_t* __restrict__ contrib, const double* __restrict__ elem_rhs,
                              double* __restrict__ rhs) {
    for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < m; row += (int64_t)gridDim.x * blockDim.x) {
        const int32_t k = diag_slot[row];
        double a = 0.;
        if (k >= 0)
        for (int32_t p = seg_start[k]; p < seg_start[k + 1]; ++p) {
            const uint32_t c = (uint32_t)contrib[p];
            const uint32_t r = c / (NL * NL);
            const int i = (int)(c - r * (NL * NL)) / NL;
            a += elem_rhs[(int64_t)r * NL + i];
        }
        rhs[row] = a;
    }
}

static int build_pattern(Context* c, const uint8_t* mask = nullptr) {
    const int nl = c->fe == TF_P2IF ? 10 : 4;
    const int64_t na = c->n_active, m = c->n_dofs;
    const int64_t ncontrib = na * nl * nl;
    if (ncontrib >= INT32_MAX) return set_err(c, TF_ERR_CAPACITY, "pattern: too many contributions for 32-bit offsets");
    TimedLaunch tl(c, TF_K_PATTERN);
    TF_TRY(ensure(c, c->row_cursor, (size_t)m + 1));
    TF_CUDA(c, cudaMemsetAsync(c->row_cursor.p, 0, sizeof(int32_t) * (size_t)(m + 1), c->stream));
    k_row_counts<<<grid_for(c, na * nl), kBlock, 0, c->stream>>>(na, nl, c->loc2glo.p, mask, c->row_cursor.p);
    ++c->launches;
    TF_TRY(ensure(c, c->rowptr, (size_t)m + 1));
    int64_t total = 0;
    // bucket starts -> rowptr buffer (temporarily)
    TF_TRY(exclusive_scan_i32_to_i32(c, c->row_cursor.p, c->rowptr.p, m, &total));
    TF_CUDA(c, cudaMemsetAsync(c->row_cursor.p, 0, sizeof(int32_t) * (size_t)(m + 1), c->stream));
    TF_TRY(ensure(c, c->contrib, (size_t)ncontrib + 1));
    k_bucket<<<grid_for(c, ncontrib), kBlock, 0, c->stream>>>(na, nl, c->loc2glo.p, mask, c->rowptr.p, c->row_cursor.p,
                                                              c->contrib.p);
    ++c->launches;
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    // unique counts into row_cursor
    k_row_sort<<<grid_for(c, m, 128, 16), 128, 0, c->stream>>>(m, c->rowptr.p, c->contrib.p, c->row_cursor.p,
                                                                 c->status.p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st) return set_err(c, st, "pattern: a matrix row has more than 1024 element contributions");
    // keep bucket starts in seg_start's tail? copy them to a separate array
    DBuf<int32_t> bstart;
    TF_TRY(ensure(c, bstart, (size_t)m + 1));
    TF_CUDA(c, cudaMemcpyAsync(bstart.p, c->rowptr.p, sizeof(int32_t) * (size_t)(m + 1), cudaMemcpyDeviceToDevice,
                               c->stream));
    int64_t nnz = 0;
    TF_TRY(exclusive_scan_i32_to_i32(c, c->row_cursor.p, c->rowptr.p, m, &nnz));
    TF_TRY(ensure(c, c->colind, (size_t)(nnz > 0 ? nnz : 1)));
    TF_TRY(ensure(c, c->seg_start, (size_t)nnz + 1));
    TF_TRY(ensure(c, c->diag_slot, (size_t)(m > 0 ? m : 1)));
    TF_CUDA(c, cudaMemsetAsync(c->diag_slot.p, 0xff, sizeof(int32_t) * (size_t)(m > 0 ? m : 1), c->stream));
    k_row_emit<<<grid_for(c, m, 128, 16), 128, 0, c->stream>>>(m, bstart.p, c->contrib.p, c->rowptr.p, c->colind.p,
                                                                 c->seg_start.p, c->diag_slot.p);
    ++c->launches;
    int32_t tot32 = (int32_t)total;  // contributions actually bucketed
    TF_CUDA(c, cudaMemcpyAsync(c->seg_start.p + nnz, &tot32, sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    release(bstart);
    TF_CUDA(c, cudaGetLastError());
    const int64_t gen = ++c->pattern_counter;
    for (int f = 0; f < TF_NUM_MATS; ++f) {
        if (!is_form_handle(f)) continue;
        CSR& A = c->mats[f];
        A.m = m;
        A.nnz = nnz;
        A.rowptr = c->rowptr.p;
        A.colind = c->colind.p;
        A.pattern_gen = gen;
        A.vals = nullptr;  // values of the old pattern: every form is assembled again
        ++A.version;
    }
    c->pattern_dof_version = mask ? -1 : c->dof_version;  // a masked pattern is not the DistributeDOFs one
    return TF_OK;
}

int setup_fe_system(Context* c, unsigned forms, int rhs_kind, const double* rhs_par, int npar) {
    if (!c->fe) return set_err(c, TF_ERR_BAD_INPUT, "setup_fe_system: distribute DOFs first");
    if (c->legacy_numbering)
        return set_err(c, TF_ERR_BAD_INPUT, "setup_fe_system: needs a DistributeDOFs numbering, not the legacy one");
    if (forms == 0 && rhs_kind == TF_RHS_NONE) return TF_OK;
    if (forms & ~(0xFu | (1u << TF_FORM_N))) return set_err(c, TF_ERR_BAD_INPUT, "setup_fe_system: unknown form bits");
    const bool p2 = c->fe == TF_P2IF;
    if (p2 && (forms & (1u << TF_FORM_LAPM)))
        return set_err(c, TF_ERR_BAD_INPUT, "setup_fe_system: LaplaceM is a P1 form");
    const bool wantN = forms & (1u << TF_FORM_N);
    if (wantN && p2) return set_err(c, TF_ERR_BAD_INPUT, "setup_fe_system: N_P1P1 is a P1 form");
    if (wantN && !c->has_wind) return set_err(c, TF_ERR_BAD_INPUT, "setup_fe_system: N_P1P1 needs tf_wind_upload");
    TF_TRY(ensure_tables(c));
    const int nl = p2 ? 10 : 4, nsym = nl * (nl + 1) / 2;
    const int64_t na = c->n_active, m = c->n_dofs;
    if (c->pattern_dof_version != c->dof_version) TF_TRY(build_pattern(c));
    RhsPar R{};
    R.kind = rhs_kind;
    for (int i = 0; i < npar && i < 8; ++i) R.p[i] = rhs_par[i];
    if (rhs_kind == TF_RHS_SPHERE_XYZ && npar < 5) return set_err(c, TF_ERR_BAD_INPUT, "rhs: 5 parameters needed");
    if (rhs_kind == TF_RHS_CONST && npar < 1) return set_err(c, TF_ERR_BAD_INPUT, "rhs: 1 parameter needed");
    TF_TRY(ensure(c, c->elem, (size_t)TF_NUM_FORMS * (size_t)(na > 0 ? na : 1) * nsym));
    TF_TRY(ensure(c, c->elem_rhs, (size_t)(na > 0 ? na : 1) * nl));
    const double* chi = nullptr;
    if (forms & (1u << TF_FORM_LAPM)) {
        if (c->vecs[TF_VEC_CHI].n == (size_t)m && m > 0) chi = c->vecs[TF_VEC_CHI].p;
    }
    if (wantN) TF_TRY(ensure(c, c->elem_n, (size_t)(na > 0 ? na : 1) * 16));
    AsmArgs A{c->mesh, c->ls_vert.p, c->ls_edge.p, na, c->active.p, c->loc2glo.p, forms, R, chi, chi ? 1 : 0,
              c->elem.p, c->elem_rhs.p, c->status.p, c->wind_v.p, c->wind_e.p, wantN ? c->elem_n.p : nullptr};
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    if (na > 0) {
        TimedLaunch tl(c, TF_K_ASSEMBLE);
        const int blocks = grid_for(c, (na + kAsmWarps - 1) / kAsmWarps, 1, 8);
        const bool pair = p2 && !c->asm_fp64 && !(forms & ~((1u << TF_FORM_M) | (1u << TF_FORM_A) | (1u << TF_FORM_CN))) &&
                          (rhs_kind == TF_RHS_NONE || rhs_kind == TF_RHS_CONST || rhs_kind == TF_RHS_SPHERE_XYZ);
        if (pair) {
            TF_TRY(ensure_tables_ff(c));
            const size_t sm = sizeof(AsmPairSmem) * kAsmWarps;
            TF_CUDA(c, cudaFuncSetAttribute(k_assemble_p2_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            // per chunk of active tets: the per-tet records (one thread per tet), then the forms (warp per tet)
            const int64_t chunk = std::min<int64_t>(na, kPrepChunk);
            TF_TRY(ensure(c, c->prep1, (size_t)chunk * sizeof(TetPrep)));
            A.prep = c->prep1.p;
            for (int64_t c0 = 0; c0 < na; c0 += chunk) {
                A.c0 = c0;
                A.c1 = std::min<int64_t>(na, c0 + chunk);
                const int64_t n = A.c1 - A.c0;
                TF_TRY(prep_order(c, A, chunk));
                k_prep_tets<false><<<grid_for(c, n, 128), 128, 0, c->stream>>>(A);
                k_assemble_p2_pair<<<grid_for(c, (n + kAsmWarps - 1) / kAsmWarps, 1, 8), 32 * kAsmWarps, sm,
                                     c->stream>>>(A);
                c->launches += 2;
            }
            --c->launches;  // counted per chunk above
        } else if (!p2 && !c->asm_fp64 && !(forms & ~((1u << TF_FORM_M) | (1u << TF_FORM_A) | (1u << TF_FORM_CN))) &&
                   (rhs_kind == TF_RHS_NONE || rhs_kind == TF_RHS_CONST || rhs_kind == TF_RHS_SPHERE_XYZ)) {
            TF_TRY(ensure_tables_ff(c));
            const size_t sm = sizeof(AsmPair1Smem) * kAsmWarps;
            TF_CUDA(c, cudaFuncSetAttribute(k_assemble_p1_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            // per chunk of active tets: the per-tet records (one thread per tet), then the forms (warp per tet)
            const int64_t chunk = std::min<int64_t>(na, kPrepChunk);
            TF_TRY(ensure(c, c->prep1, (size_t)chunk * sizeof(TetPrep)));
            A.prep = c->prep1.p;
            for (int64_t c0 = 0; c0 < na; c0 += chunk) {
                A.c0 = c0;
                A.c1 = std::min<int64_t>(na, c0 + chunk);
                const int64_t n = A.c1 - A.c0;
                TF_TRY(prep_order(c, A, chunk));
                k_prep_tets<true><<<grid_for(c, n, 128), 128, 0, c->stream>>>(A);
                k_assemble_p1_pair<<<grid_for(c, (n + kAsmWarps - 1) / kAsmWarps, 1, 8), 32 * kAsmWarps, sm,
                                     c->stream>>>(A);
                c->launches += 2;
            }
            --c->launches;  // counted per chunk above
        } else if (p2) {
            const size_t sm = sizeof(AsmSmem<10>) * kAsmWarps;
            TF_CUDA(c, cudaFuncSetAttribute(k_assemble<10>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            k_assemble<10><<<blocks, 32 * kAsmWarps, sm, c->stream>>>(A);
        } else {
            const size_t sm = sizeof(AsmSmem<4>) * kAsmWarps;
            TF_CUDA(c, cudaFuncSetAttribute(k_assemble<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            k_assemble<4><<<blocks, 32 * kAsmWarps, sm, c->stream>>>(A);
        }
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
    }
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st == TF_ERR_ZERO_PATTERN)
        return set_err(c, st, "RefPatchCL::instance: found a full body in the zero level set, grid is too coarse");
    if (st) return set_err(c, st, "assembly failed");
    // values
    double* v[4] = {nullptr, nullptr, nullptr, nullptr};
    const int64_t nnz = c->mats[0].nnz;
    for (int f = 0; f < TF_NUM_FORMS; ++f) {
        if (!(forms & (1u << f))) continue;
        TF_TRY(ensure(c, c->mat_vals[f], (size_t)(nnz > 0 ? nnz : 1)));
        c->mats[f].vals = c->mat_vals[f].p;
        ++c->mats[f].version;
        v[f] = c->mats[f].vals;
    }
    double* vN = nullptr;
    if (wantN) {
        TF_TRY(ensure(c, c->mat_vals[TF_FORM_N], (size_t)(nnz > 0 ? nnz : 1)));
        c->mats[TF_FORM_N].vals = vN = c->mat_vals[TF_FORM_N].p;
        ++c->mats[TF_FORM_N].version;
    }
    if (nnz > 0) {
        TimedLaunch tl(c, TF_K_SCATTER);
        if (p2)
            k_scatter<10><<<grid_for(c, nnz), kBlock, 0, c->stream>>>(nnz, c->seg_start.p, c->contrib.p, na, c->elem.p,
                                                                       forms, v[0], v[1], v[2], v[3]);
        else
            k_scatter<4><<<grid_for(c, nnz), kBlock, 0, c->stream>>>(nnz, c->seg_start.p, c->contrib.p, na, c->elem.p,
                                                                      forms, v[0], v[1], v[2], v[3], c->elem_n.p, vN);
        ++c->launches;
        if (rhs_kind != TF_RHS_NONE) {
            TF_TRY(ensure(c, c->vecs[TF_VEC_RHS], (size_t)m));
            if (p2)
                k_scatter_rhs<10><<<grid_for(c, m), kBlock, 0, c->stream>>>(m, c->diag_slot.p, c->seg_start.p, c->contrib.p,
                                                                             c->elem_rhs.p, c->vecs[TF_VEC_RHS].p);
            else
                k_scatter_rhs<4><<<grid_for(c, m), kBlock, 0, c->stream>>>(m, c->diag_slot.p, c->seg_start.p, c->contrib.p,
                                                                            c->elem_rhs.p, c->vecs[TF_VEC_RHS].p);
            ++c->launches;
        }
        TF_CUDA(c, cudaGetLastError());
    }
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    return TF_OK;
}

// ---------------------------------------------------------------------------
// isoparametric P2 forms (QuaQua mapper, quaqua.cu) into TF_FORM_M, TF_FORM_A
// and TF_VEC_RHS on the DistributeDOFs pattern
// ---------------------------------------------------------------------------
int setup_quaqua_p2(Context* c, double rhs_c, double tol, int maxiter, int* newton_max) {
    if (!c->fe) return set_err(c, TF_ERR_BAD_INPUT, "setup_quaqua_p2: distribute DOFs first");
    if (tol <= 0. || maxiter < 1) return set_err(c, TF_ERR_BAD_INPUT, "setup_quaqua_p2: tol > 0, maxiter >= 1");
    if (c->pattern_dof_version != c->dof_version) TF_TRY(build_pattern(c));
    TF_TRY(quaqua_elements(c, rhs_c, tol, maxiter, newton_max));
    const int64_t na = c->n_active, m = c->n_dofs, nnz = c->mats[0].nnz;
    double* v[2];
    for (int f = 0; f < 2; ++f) {  // TF_FORM_M, TF_FORM_A
        TF_TRY(ensure(c, c->mat_vals[f], (size_t)(nnz > 0 ? nnz : 1)));
        c->mats[f].vals = c->mat_vals[f].p;
        ++c->mats[f].version;
        v[f] = c->mats[f].vals;
    }
    TF_TRY(ensure(c, c->vecs[TF_VEC_RHS], (size_t)m));
    if (nnz > 0) {
        TimedLaunch tl(c, TF_K_SCATTER);
        k_scatter<10><<<grid_for(c, nnz), kBlock, 0, c->stream>>>(nnz, c->seg_start.p, c->contrib.p, na, c->elem.p,
                                                                   (1u << TF_FORM_M) | (1u << TF_FORM_A), v[0], v[1],
                                                                   nullptr, nullptr);
        k_scatter_rhs<10><<<grid_for(c, m), kBlock, 0, c->stream>>>(m, c->diag_slot.p, c->seg_start.p, c->contrib.p,
                                                                     c->elem_rhs.p, c->vecs[TF_VEC_RHS].p);
        c->launches += 2;
        TF_CUDA(c, cudaGetLastError());
    }
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    return TF_OK;
}

// ---------------------------------------------------------------------------
// legacy P1 interface forms of the surfactant.cpp path
// ---------------------------------------------------------------------------
// InterfacePatchCL::Sign (num/interfacePatch.h:75): |phi| < 2 eps counts as 0
__device__ inline int legacy_sign(double phi) {
    return fabs(phi) < 4.440892098500626e-16 ? 0 : (phi > 0. ? 1 : -1);
}

__device__ inline double rhs_quadratic(const double* p, const double x[3]) {
    return ((p[0] + p[1] * x[0] + p[2] * x[1] + p[3] * x[2]) + (p[4] * x[0] * x[0] + p[5] * x[1] * x[1] + p[6] * x[2] * x[2])) +
           (p[7] * x[0] * x[1] + p[8] * x[0] * x[2] + p[9] * x[1] * x[2]);
}

// Planar pieces of regular child ch: InterfacePatchCL::ComputeVerticesOfCut
// (num/interfacePatch.cpp:137-199) with linear edge roots, then
// InterfaceTriangleCL::ComputeForChild (:478-512): triangle (P,Q,R) with
// |det|, for four points also (Q,R,S) with |det| (a + b - 1) from the least-
// squares fit S - P = a (Q - P) + b (R - P); halved when the patch is a face
// shared by two children.  Returns the triangle count, -1 for a 3-D zero set.
__device__ int legacy_child_triangles(const double X[4][3], const double ls10[10], int ch, double tri[2][3][4],
                                      double det[2]) {
    const int* cv = cT.reg_child[ch];
    int ns[3] = {0, 0, 0}, sg[4];
    for (int k = 0; k < 4; ++k) {
        sg[k] = legacy_sign(ls10[cv[k]]);
        ++ns[sg[k] + 1];
    }
    if (ns[0] * ns[2] == 0 && ns[1] < 3) return 0;
    if (ns[1] == 4) return -1;
    auto bdof = [&](int v, double b[4]) {
        for (int c = 0; c < 4; ++c) b[c] = 0.;
        if (v < 4) b[v] = 1.;
        else { b[ev0(v - 4)] = 0.5; b[ev1(v - 4)] = 0.5; }
    };
    auto cdof = [&](int v, double x[3]) {
        if (v < 4) for (int c = 0; c < 3; ++c) x[c] = X[v][c];
        else for (int c = 0; c < 3; ++c) x[c] = 0.5 * (X[ev0(v - 4)][c] + X[ev1(v - 4)][c]);
    };
    double bary[4][4], pqrs[4][3];
    int np = 0;
    for (int k = 0; k < 4; ++k)
        if (sg[k] == 0) {
            bdof(cv[k], bary[np]);
            cdof(cv[k], pqrs[np]);
            ++np;
        }
    for (int e = 0; e < 6; ++e) {
        const int k0 = ev0(e), k1 = ev1(e);
        if (sg[k0] * sg[k1] < 0) {
            const int v0 = cv[k0], v1 = cv[k1];
            const double lam = ls10[v0] / (ls10[v0] - ls10[v1]);
            double b0[4], b1[4], x0[3], x1[3];
            bdof(v0, b0);
            bdof(v1, b1);
            cdof(v0, x0);
            cdof(v1, x1);
            for (int c = 0; c < 4; ++c) bary[np][c] = (1. - lam) * b0[c] + lam * b1[c];
            for (int c = 0; c < 3; ++c) pqrs[np][c] = (1. - lam) * x0[c] + lam * x1[c];
            ++np;
        }
    }
    for (int f = 0; f < 4; ++f) {  // cut lying on a face of the parent
        int on = 0;
        for (int i = 0; i < np; ++i) on += bary[i][f] < 1e-9;
        if (on == np) return 0;
    }
    if (np < 3) return 0;
    double u[3], v[3];
    for (int c = 0; c < 3; ++c) {
        u[c] = pqrs[1][c] - pqrs[0][c];
        v[c] = pqrs[2][c] - pqrs[0][c];
    }
    const double c0 = u[1] * v[2] - u[2] * v[1], c1 = u[2] * v[0] - u[0] * v[2], c2 = u[0] * v[1] - u[1] * v[0];
    double d = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    if (ns[1] >= 3) d /= 2.;
    for (int j = 0; j < 3; ++j)
        for (int c = 0; c < 4; ++c) tri[0][j][c] = bary[j][c];
    det[0] = d;
    if (np < 4) return 1;
    double w[3];
    for (int c = 0; c < 3; ++c) w[c] = pqrs[3][c] - pqrs[0][c];
    const double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2], uv = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
    const double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2], uw = u[0] * w[0] + u[1] * w[1] + u[2] * w[2];
    const double vw = v[0] * w[0] + v[1] * w[1] + v[2] * w[2];
    const double dd = uu * vv - uv * uv;
    const double aa = (uw * vv - vw * uv) / dd, bb = (vw * uu - uw * uv) / dd;
    for (int j = 0; j < 3; ++j)
        for (int c = 0; c < 4; ++c) tri[1][j][c] = bary[j + 1][c];
    det[1] = d * (aa + bb - 1.);
    return 2;
}

struct LegacySmem {
    TetGeom g;
    double gM[9], gC[9];
    double ls10[10];
    PatchSmem P;
};

struct LegacyArgs {
    MeshView M;
    const double* lsv;
    const double* lse;
    int64_t n;               // tets in the list
    const int32_t* tets;
    double alpha, D;
    int want_rhs;
    double fp[10];
    double* elem;            // [form][n][10]
    double* elem_rhs;        // [n][4]
    uint8_t* nonempty;       // [n]
    int* status;
};

// warp per tet: LocalInterfaceMassP1CL (Quad2_2D composite rule on the
// lattice-2 patch; diagonal unscaled, off-diagonal x alpha,
// surfactant/ifacetransp.h:881-906), LocalLaplaceBeltramiP1CL (facet
// normals, D/2 sum |det_f| without halving on lattice faces, :1657-1695) on
// one lane per facet, and the SetupInterfaceRhsP1 contributions
// (surfactant/ifacetransp.cpp:515-563) on one lane per regular child;
// lane sums combined by a fixed shuffle tree.
__global__ void __launch_bounds__(32 * kAsmWarps) k_assemble_legacy(LegacyArgs A) {
    __shared__ LegacySmem smem[kAsmWarps];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    LegacySmem& S = smem[wib];
    const int64_t nwarps = (int64_t)gridDim.x * kAsmWarps;
    for (int64_t r = (int64_t)blockIdx.x * kAsmWarps + wib; r < A.n; r += nwarps) {
        const int32_t t = A.tets[r];
        int32_t v[4], e[6];
        mesh_tet(A.M, t, v, e);
        if (lane < 4) {
            double x[3];
            mesh_coord(A.M, v[lane], x);
            for (int c = 0; c < 3; ++c) S.g.X[lane][c] = x[c];
            S.ls10[lane] = A.lsv[v[lane]];
        } else if (lane < 10) {
            S.ls10[lane] = A.lse[e[lane - 4]];
        }
        __syncwarp();
        warp_tet_geometry(S.g, S.ls10, S.gM, S.gC, lane);
        double ls10[10];
        for (int k = 0; k < 10; ++k) ls10[k] = S.ls10[k];
        const int nf = warp_patch(ls10, S.g.X, S.P, lane, A.status, t);
        double mq[10], lq[10], rq[4];
        for (int k = 0; k < 10; ++k) mq[k] = lq[k] = 0.;
        for (int k = 0; k < 4; ++k) rq[k] = 0.;
        if (lane < nf) {
            double w[3][3];
            for (int j = 0; j < 3; ++j)
                for (int c = 0; c < 3; ++c)
                    w[j][c] = S.g.X[0][c] * S.P.fb[lane][j][0] + S.g.X[1][c] * S.P.fb[lane][j][1] +
                              S.g.X[2][c] * S.P.fb[lane][j][2] + S.g.X[3][c] * S.P.fb[lane][j][3];
            double u[3], vv[3];
            for (int c = 0; c < 3; ++c) {
                u[c] = w[1][c] - w[0][c];
                vv[c] = w[2][c] - w[0][c];
            }
            const double cr[3] = {u[1] * vv[2] - u[2] * vv[1], u[2] * vv[0] - u[0] * vv[2], u[0] * vv[1] - u[1] * vv[0]};
            const double ad = sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
            const double wq = ad * (S.P.bnd[lane] ? 0.5 : 1.);
            for (int q = 0; q < 4; ++q) {
                double b[4];
                for (int c = 0; c < 4; ++c)
                    b[c] = S.P.fb[lane][0][c] * cT.qq2_node[q][0] + S.P.fb[lane][1][c] * cT.qq2_node[q][1] +
                           S.P.fb[lane][2][c] * cT.qq2_node[q][2];
                const double wt = wq * cT.qq2_w[q];
                for (int k = 0; k < 10; ++k) mq[k] += wt * (b[cT.sym4_i[k]] * b[cT.sym4_j[k]]);
            }
            if (ad > 0.) {
                const double n[3] = {cr[0] / ad, cr[1] / ad, cr[2] / ad};
                double pq[4][3];
                for (int i = 0; i < 4; ++i) {
                    const double gn = S.g.gl[i][0] * n[0] + S.g.gl[i][1] * n[1] + S.g.gl[i][2] * n[2];
                    for (int c = 0; c < 3; ++c) pq[i][c] = S.g.gl[i][c] - gn * n[c];
                }
                for (int k = 0; k < 10; ++k) {
                    const int i = cT.sym4_i[k], j = cT.sym4_j[k];
                    lq[k] += (pq[i][0] * pq[j][0] + pq[i][1] * pq[j][1] + pq[i][2] * pq[j][2]) * ad;
                }
            }
        }
        if (A.want_rhs && lane < 8) {
            const int s0 = legacy_sign(ls10[0]);
            bool inter = false;
            for (int k = 1; k < 10; ++k) inter |= legacy_sign(ls10[k]) != s0;
            if (inter) {
                double tri[2][3][4], det[2];
                const int ntr = legacy_child_triangles(S.g.X, ls10, lane, tri, det);
                if (ntr < 0) set_status(A.status, TF_ERR_ZERO_PATTERN, t);
                for (int tt = 0; tt < ntr; ++tt)
                    for (int q = 0; q < 7; ++q) {
                        double b[4], x[3];
                        for (int c = 0; c < 4; ++c)
                            b[c] = tri[tt][0][c] * cT.q2_node[q][0] + tri[tt][1][c] * cT.q2_node[q][1] +
                                   tri[tt][2][c] * cT.q2_node[q][2];
                        for (int c = 0; c < 3; ++c)
                            x[c] = S.g.X[0][c] * b[0] + S.g.X[1][c] * b[1] + S.g.X[2][c] * b[2] + S.g.X[3][c] * b[3];
                        const double fx = rhs_quadratic(A.fp, x);
                        for (int i = 0; i < 4; ++i) rq[i] += (det[tt] * cT.q2_w[q]) * (fx * b[i]);
                    }
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            for (int k = 0; k < 10; ++k) {
                mq[k] += __shfl_xor_sync(0xffffffffu, mq[k], o);
                lq[k] += __shfl_xor_sync(0xffffffffu, lq[k], o);
            }
            for (int k = 0; k < 4; ++k) rq[k] += __shfl_xor_sync(0xffffffffu, rq[k], o);
        }
        if (lane < 10) {
            const int k = lane;
            const bool diag = cT.sym4_i[k] == cT.sym4_j[k];
            double mv = 0., lv = 0.;
            for (int kk = 0; kk < 10; ++kk)
                if (kk == k) {
                    mv = mq[kk];
                    lv = lq[kk];
                }
            A.elem[((int64_t)TF_FORM_M * A.n + r) * 10 + k] = diag ? mv : A.alpha * mv;
            A.elem[((int64_t)TF_FORM_A * A.n + r) * 10 + k] = (A.D * 0.5) * lv;
        }
        if (lane < 4) {
            double rv = 0.;
            for (int i = 0; i < 4; ++i)
                if (i == lane) rv = rq[i];
            A.elem_rhs[r * 4 + lane] = rv;
        }
        if (lane == 0) {
            A.nonempty[r] = nf > 0;
            // a rhs piece on a tet whose patch is empty (values within 2 eps
            // of zero) has no slot in the pattern: counted for a fix-up pass
            if (nf == 0 && (rq[0] != 0. || rq[1] != 0. || rq[2] != 0. || rq[3] != 0.)) atomicAdd(A.status + 2, 1);
        }
        __syncwarp();
    }
}

// rhs pieces of tets outside the masked pattern, added in tet order by one
// thread (runs only when the assembly counted such tets)
__global__ void k_legacy_rhs_stray(int64_t n, const uint8_t* __restrict__ nonempty, const int32_t* __restrict__ l2g,
                                   const double* __restrict__ elem_rhs, double* __restrict__ rhs) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    for (int64_t r = 0; r < n; ++r) {
        if (nonempty[r]) continue;
        for (int i = 0; i < 4; ++i) {
            const int32_t d = l2g[4 * r + i];
            if (d >= 0) rhs[d] += elem_rhs[4 * r + i];
        }
    }
}

int setup_legacy_p1(Context* c, double alpha, double D, const double* fpar, int64_t* nnz_out) {
    if (c->fe != TF_P1IF) return set_err(c, TF_ERR_BAD_INPUT, "legacy forms: a P1 interface numbering is required");
    TF_TRY(ensure_tables(c));
    const int64_t na = c->n_active, m = c->n_dofs;
    TF_TRY(ensure(c, c->elem, (size_t)TF_NUM_FORMS * (size_t)(na > 0 ? na : 1) * 10));
    TF_TRY(ensure(c, c->elem_rhs, (size_t)(na > 0 ? na : 1) * 4));
    TF_TRY(ensure(c, c->legacy_mask, (size_t)(na > 0 ? na : 1)));
    LegacyArgs A{};
    A.M = c->mesh;
    A.lsv = c->ls_vert.p;
    A.lse = c->ls_edge.p;
    A.n = na;
    A.tets = c->active.p;
    A.alpha = alpha;
    A.D = D;
    A.want_rhs = fpar != nullptr;
    for (int i = 0; i < 10; ++i) A.fp[i] = fpar ? fpar[i] : 0.;
    A.elem = c->elem.p;
    A.elem_rhs = c->elem_rhs.p;
    A.nonempty = c->legacy_mask.p;
    A.status = c->status.p;
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    if (na > 0) {
        TimedLaunch tl(c, TF_K_ASSEMBLE);
        k_assemble_legacy<<<grid_for(c, (na + kAsmWarps - 1) / kAsmWarps, 1, 8), 32 * kAsmWarps, 0, c->stream>>>(A);
        ++c->launches;
        TF_CUDA(c, cudaGetLastError());
    }
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st == TF_ERR_ZERO_PATTERN)
        return set_err(c, st, "legacy forms: zero level set of positive volume on a lattice sub-tet or child");
    if (st) return set_err(c, st, "legacy forms failed");
    const int stray = c->h_status[2];
    TF_TRY(build_pattern(c, c->legacy_mask.p));
    const int64_t nnz = c->mats[0].nnz;
    double* v[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int f : {TF_FORM_M, TF_FORM_A}) {
        TF_TRY(ensure(c, c->mat_vals[f], (size_t)(nnz > 0 ? nnz : 1)));
        c->mats[f].vals = c->mat_vals[f].p;
        ++c->mats[f].version;
        v[f] = c->mats[f].vals;
    }
    for (int f : {TF_FORM_CN, TF_FORM_LAPM, TF_FORM_N}) c->mats[f].vals = nullptr;  // not part of this pattern
    if (nnz > 0) {
        TimedLaunch tl(c, TF_K_SCATTER);
        const unsigned forms = (1u << TF_FORM_M) | (1u << TF_FORM_A);
        k_scatter<4><<<grid_for(c, nnz), kBlock, 0, c->stream>>>(nnz, c->seg_start.p, c->contrib.p, na, c->elem.p, forms,
                                                                  v[0], v[1], v[2], v[3]);
        ++c->launches;
    }
    if (fpar) {
        TF_TRY(ensure(c, c->vecs[TF_VEC_RHS], (size_t)m));
        if (m > 0) {
            k_scatter_rhs<4><<<grid_for(c, m), kBlock, 0, c->stream>>>(m, c->diag_slot.p, c->seg_start.p, c->contrib.p,
                                                                        c->elem_rhs.p, c->vecs[TF_VEC_RHS].p);
            ++c->launches;
        }
        if (stray > 0) {
            k_legacy_rhs_stray<<<1, 32, 0, c->stream>>>(na, c->legacy_mask.p, c->loc2glo.p, c->elem_rhs.p,
                                                        c->vecs[TF_VEC_RHS].p);
            ++c->launches;
        }
    }
    TF_CUDA(c, cudaGetLastError());
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    if (nnz_out) *nnz_out = nnz;
    return TF_OK;
}

__global__ void k_fill_i32_asm(int32_t* p, int64_t n, int32_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = v;
}
__global__ void k_mark_owned_asm(int64_t n, const int32_t* __restrict__ keys, int32_t* __restrict__ owned) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (keys[i] != INT_MAX) owned[keys[i]] = 1;
}
__global__ void k_assign_asm(int64_t n, const int32_t* __restrict__ keys, const int32_t* __restrict__ rank,
                             int32_t* __restrict__ dof) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dof[i] = keys[i] != INT_MAX ? rank[keys[i]] : -1;
}

// ---------------------------------------------------------------------------
// patch topology in the reference's own numbering (for parity checks):
// SPatchCL<3>::make_patch<MergeCutPolicyCL> (geom/subtriangulation.tpp:191-228)
// replayed per tet -- cut vertices numbered in discovery order, copied zero
// vertices after them, facets in sub-tet order.
// ---------------------------------------------------------------------------
__global__ void k_patch_dump(MeshView M, const double* __restrict__ lsv, const double* __restrict__ lse,
                             const int32_t* __restrict__ tets, int64_t count, int32_t* __restrict__ nf_out,
                             int32_t* __restrict__ facets, int32_t* __restrict__ bnd_out, int32_t* __restrict__ nv_out,
                             double* __restrict__ verts, int* status) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < count; r += (int64_t)gridDim.x * blockDim.x) {
        int32_t v[4], e[6];
        mesh_tet(M, tets[r], v, e);
        double ls10[10], lat[10];
        for (int k = 0; k < 4; ++k) ls10[k] = lsv[v[k]];
        for (int k = 0; k < 6; ++k) ls10[4 + k] = lse[e[k]];
        for (int k = 0; k < 10; ++k) lat[cP2OnLat[k]] = ls10[k];
        int cut_a[32], cut_b[32], ncut = 0;
        int copied[10];
        for (int k = 0; k < 10; ++k) copied[k] = -1;
        int zero_lat[10], nzero = 0;
        int zf[48], zj[48], nz = 0;
        int nf = 0;
        int32_t* F = facets + r * 48;
        for (int s = 0; s < 8; ++s) {
            int pat = 0;
            for (int k = 0; k < 4; ++k) {
                const double x = lat[cT.lat_t[s][k]];
                pat += ((x > 0.) - (x < 0.) + 1) * (k == 0 ? 1 : k == 1 ? 3 : k == 2 ? 9 : 27);
            }
            const int n = cT.pat_nf[pat];
            if (n < 0) {
                set_status(status, TF_ERR_ZERO_PATTERN, tets[r]);
                break;
            }
            for (int f = 0; f < n; ++f, ++nf) {
                bnd_out[r * 16 + nf] = cT.pat_bnd[pat];
                for (int j = 0; j < 3; ++j) {
                    const int ext = cT.pat_f[pat][f][j];
                    if (ext < 4) {
                        const int L = cT.lat_t[s][ext];
                        if (copied[L] < 0) {
                            copied[L] = nzero;
                            zero_lat[nzero++] = L;
                        }
                        F[3 * nf + j] = copied[L];
                        zf[nz] = nf;
                        zj[nz] = j;
                        ++nz;
                    } else {
                        const int a = cT.can_a[s][ext - 4], b = cT.can_b[s][ext - 4];
                        int id = -1;
                        for (int q = 0; q < ncut; ++q)
                            if (cut_a[q] == a && cut_b[q] == b) id = q;
                        if (id < 0) {
                            id = ncut++;
                            cut_a[id] = a;
                            cut_b[id] = b;
                        }
                        F[3 * nf + j] = id;
                    }
                }
            }
        }
        for (int u = 0; u < nz; ++u) F[3 * zf[u] + zj[u]] += ncut;
        nf_out[r] = nf;
        nv_out[r] = ncut + nzero;
        double* V = verts + r * 40 * 4;
        for (int q = 0; q < ncut; ++q) cut_point(lat, cut_a[q], cut_b[q], V + 4 * q);
        for (int q = 0; q < nzero; ++q)
            for (int c2 = 0; c2 < 4; ++c2) V[4 * (ncut + q) + c2] = cT.lat_v[zero_lat[q]][c2];
    }
}

int patch_dump(Context* c, const int32_t* tets, int64_t count, int32_t* nf, int32_t* facets, int32_t* bnd,
               int32_t* nverts, double* verts) {
    if (!c->has_mesh || !c->has_ls) return set_err(c, TF_ERR_BAD_INPUT, "patches: mesh and level set required");
    if (count < 0 || (count > 0 && !tets)) return set_err(c, TF_ERR_BAD_INPUT, "patches: tet ids required");
    for (int64_t i = 0; i < count; ++i)
        if (tets[i] < 0 || tets[i] >= c->mesh.nt) return set_err(c, TF_ERR_BAD_INPUT, "patches: tet id out of range");
    TF_TRY(ensure_tables(c));
    if (count == 0) return TF_OK;
    DBuf<int32_t> i32;
    DBuf<double> f64;
    TF_TRY(ensure(c, i32, (size_t)count * (1 + 48 + 16 + 1 + 1)));
    TF_TRY(ensure(c, f64, (size_t)count * 160));
    int32_t* dtet = i32.p + count * 66;
    TF_CUDA(c, cudaMemcpy(dtet, tets, sizeof(int32_t) * count, cudaMemcpyHostToDevice));
    int32_t* dnf = i32.p;
    int32_t* dfac = dnf + count;
    int32_t* dbnd = dfac + count * 48;
    int32_t* dnv = dbnd + count * 16;
    TF_CUDA(c, cudaMemsetAsync(i32.p, 0, sizeof(int32_t) * (size_t)count * 66, c->stream));
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    k_patch_dump<<<grid_for(c, count), 128, 0, c->stream>>>(c->mesh, c->ls_vert.p, c->ls_edge.p, dtet, count,
                                                            dnf, dfac, dbnd, dnv, f64.p, c->status.p);
    ++c->launches;
    TF_CUDA(c, cudaGetLastError());
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st == 0) {
        if (nf) TF_CUDA(c, cudaMemcpy(nf, dnf, sizeof(int32_t) * count, cudaMemcpyDeviceToHost));
        if (facets) TF_CUDA(c, cudaMemcpy(facets, dfac, sizeof(int32_t) * count * 48, cudaMemcpyDeviceToHost));
        if (bnd) TF_CUDA(c, cudaMemcpy(bnd, dbnd, sizeof(int32_t) * count * 16, cudaMemcpyDeviceToHost));
        if (nverts) TF_CUDA(c, cudaMemcpy(nverts, dnv, sizeof(int32_t) * count, cudaMemcpyDeviceToHost));
        if (verts) TF_CUDA(c, cudaMemcpy(verts, f64.p, sizeof(double) * count * 160, cudaMemcpyDeviceToHost));
    }
    release(i32);
    release(f64);
    if (st) return set_err(c, st, "RefPatchCL::instance: found a full body in the zero level set");
    return TF_OK;
}

// ---------------------------------------------------------------------------
// legacy numbering: CreateNumbOnInterfaceVertex (misc/problem.cpp:443-505)
// A vertex gets its number at the first tet (triangulation order) whose patch
// carries a Quad2 integral of lambda_i^2 above omit_bound * (6|T|)^{4/3};
// the key t*4 + i of that first qualifying (tet, vertex) orders the numbers.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(32 * kAsmWarps) k_legacy_touch(MeshView M, const double* __restrict__ lsv,
                                                                const double* __restrict__ lse, int64_t n_cand,
                                                                const int32_t* __restrict__ cand, double omit_bound,
                                                                int32_t* __restrict__ keys, uint8_t* __restrict__ nonempty,
                                                                int* status) {
    __shared__ PatchSmem Ps[kAsmWarps];
    __shared__ double Xs[kAsmWarps][4][3];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    PatchSmem& P = Ps[wib];
    for (int64_t r = (int64_t)blockIdx.x * kAsmWarps + wib; r < n_cand; r += (int64_t)gridDim.x * kAsmWarps) {
        const int32_t t = cand[r];
        int32_t v[4], e[6];
        mesh_tet(M, t, v, e);
        double ls10[10];
        for (int k = 0; k < 4; ++k) ls10[k] = lsv[v[k]];
        for (int k = 0; k < 6; ++k) ls10[4 + k] = lse[e[k]];
        if (lane < 4) {
            double x[3];
            mesh_coord(M, v[lane], x);
            for (int c2 = 0; c2 < 3; ++c2) Xs[wib][lane][c2] = x[c2];
        }
        __syncwarp();
        double X[4][3];
        for (int k = 0; k < 4; ++k)
            for (int c2 = 0; c2 < 3; ++c2) X[k][c2] = Xs[wib][k][c2];
        const int nf = warp_patch(ls10, X, P, lane, status, t);
        if (lane == 0) nonempty[r] = nf > 0;
        if (nf == 0) {
            __syncwarp();
            continue;
        }
        // 6|T| = |det J|
        double M3[3][3];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) M3[j][i] = X[i + 1][j] - X[0][j];
        const double det = M3[0][0] * (M3[1][1] * M3[2][2] - M3[1][2] * M3[2][1]) -
                           M3[0][1] * (M3[1][0] * M3[2][2] - M3[1][2] * M3[2][0]) +
                           M3[0][2] * (M3[1][0] * M3[2][1] - M3[1][1] * M3[2][0]);
        const double limit = omit_bound < 0. ? 0. : omit_bound * pow(fabs(det), 4. / 3.);
        double acc[4] = {0, 0, 0, 0};
        for (int p = lane; p < 4 * nf; p += 32) {
            const int f = p >> 2, q = p & 3;
            double b[4];
            for (int c2 = 0; c2 < 4; ++c2)
                b[c2] = P.fb[f][0][c2] * cT.qq2_node[q][0] + P.fb[f][1][c2] * cT.qq2_node[q][1] +
                        P.fb[f][2][c2] * cT.qq2_node[q][2];
            const double w = P.fw[f] * cT.qq2_w[q];
            double h[10];
            for (int i = 0; i < 4; ++i) h[i] = b[i] * (2. * b[i] - 1.);
            for (int k = 0; k < 6; ++k) h[4 + k] = 4. * b[ev0(k)] * b[ev1(k)];
            for (int i = 0; i < 4; ++i) {
                // lambda_i^2 as a P2 function: 1 at vertex i, 1/4 on the edges at i
                double val = 0.;
                for (int k = 0; k < 10; ++k) {
                    const double ck = k < 4 ? (k == i ? 1. : 0.) : ((ev0(k - 4) == i || ev1(k - 4) == i) ? 0.25 : 0.);
                    val += ck * h[k];
                }
                acc[i] += w * val;
            }
        }
        for (int i = 0; i < 4; ++i)
            for (int o = 16; o > 0; o >>= 1) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], o);
        if (lane < 4 && acc[lane] > limit) atomicMin(&keys[v[lane]], (int32_t)(t * 4 + lane));
        __syncwarp();
    }
}

__global__ void k_legacy_active(MeshView M, int64_t n_cand, const int32_t* __restrict__ cand,
                                const uint8_t* __restrict__ nonempty, const int32_t* __restrict__ keys,
                                int32_t* __restrict__ act_flag) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n_cand; r += (int64_t)gridDim.x * blockDim.x) {
        int a = 0;
        if (nonempty[r]) {
            const int32_t t = cand[r];
            int32_t v[4];
            mesh_tet(M, t, v, nullptr);
            for (int i = 0; i < 4; ++i) {
                const int32_t k = keys[v[i]];
                if (k != INT_MAX && k / 4 <= t) a = 1;
            }
        }
        act_flag[r] = a;
    }
}

int compact_active(Context* c, int64_t* n_active);

// local-to-global map of the cut tets under the legacy numbering (-1: vertex not numbered)
__global__ void k_legacy_l2g(MeshView M, int64_t n, const int32_t* __restrict__ tets,
                             const int32_t* __restrict__ dof_vert, int32_t* __restrict__ l2g) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        int32_t v[4];
        mesh_tet(M, tets[r], v, nullptr);
        for (int i = 0; i < 4; ++i) l2g[4 * r + i] = dof_vert[v[i]];
    }
}

int numb_on_interface_p1(Context* c, double omit_bound) {
    if (!c->has_mesh || !c->has_ls) return set_err(c, TF_ERR_BAD_INPUT, "numbering: mesh and level set required");
    TF_TRY(ensure_tables(c));
    const MeshView& M = c->mesh;
    if (M.nt * 4 >= INT_MAX) return set_err(c, TF_ERR_CAPACITY, "numbering: too many tets for 32-bit keys");
    c->fe = 0;
    // cut tets (distance == 0 on the lattice values) -> candidate list
    TF_TRY(distribute_dofs(c, TF_P1IF, 0.0));
    const int64_t n_cand = c->n_active;
    DBuf<int32_t> cand;
    DBuf<uint8_t> nonempty;
    TF_TRY(ensure(c, cand, (size_t)(n_cand > 0 ? n_cand : 1)));
    TF_TRY(ensure(c, nonempty, (size_t)(n_cand > 0 ? n_cand : 1)));
    TF_CUDA(c, cudaMemcpyAsync(cand.p, c->active.p, sizeof(int32_t) * n_cand, cudaMemcpyDeviceToDevice, c->stream));
    TF_TRY(ensure(c, c->keys_v, (size_t)M.nv));
    TF_TRY(ensure(c, c->dof_vert, (size_t)M.nv));
    k_fill_i32_asm<<<grid_for(c, M.nv), kBlock, 0, c->stream>>>(c->keys_v.p, M.nv, INT_MAX);
    ++c->launches;
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    if (n_cand > 0) {
        k_legacy_touch<<<grid_for(c, (n_cand + kAsmWarps - 1) / kAsmWarps, 1, 8), 32 * kAsmWarps, 0, c->stream>>>(
            M, c->ls_vert.p, c->ls_edge.p, n_cand, cand.p, omit_bound, c->keys_v.p, nonempty.p, c->status.p);
        ++c->launches;
    }
    int st = 0;
    TF_TRY(sync_status(c, &st));
    if (st) {
        release(cand);
        release(nonempty);
        return set_err(c, st, "legacy numbering: all-zero sign pattern on a lattice sub-tet");
    }
    // ranks over the key space t*4+i
    const int64_t nkeys = M.nt * 4;
    TF_TRY(ensure(c, c->owner, (size_t)nkeys + 1));
    TF_CUDA(c, cudaMemsetAsync(c->owner.p, 0, sizeof(int32_t) * (size_t)(nkeys + 1), c->stream));
    k_mark_owned_asm<<<grid_for(c, M.nv), kBlock, 0, c->stream>>>(M.nv, c->keys_v.p, c->owner.p);
    ++c->launches;
    DBuf<int32_t> rank;
    TF_TRY(ensure(c, rank, (size_t)nkeys + 1));
    int64_t ndofs = 0;
    TF_TRY(exclusive_scan_i32_to_i32(c, c->owner.p, rank.p, nkeys, &ndofs));
    k_assign_asm<<<grid_for(c, M.nv), kBlock, 0, c->stream>>>(M.nv, c->keys_v.p, rank.p, c->dof_vert.p);
    ++c->launches;
    // active tets: a cut tet with a non-empty patch that touches a numbered vertex
    TF_TRY(ensure(c, c->scratch, (size_t)M.nt * sizeof(int32_t)));
    TF_CUDA(c, cudaMemsetAsync(c->scratch.p, 0, sizeof(int32_t) * (size_t)M.nt, c->stream));
    DBuf<int32_t> flag;
    TF_TRY(ensure(c, flag, (size_t)(n_cand > 0 ? n_cand : 1)));
    if (n_cand > 0) {
        k_legacy_active<<<grid_for(c, n_cand), kBlock, 0, c->stream>>>(M, n_cand, cand.p, nonempty.p, c->keys_v.p, flag.p);
        ++c->launches;
    }
    int64_t na = 0;
    TF_TRY(exclusive_scan_i32_to_i32(c, flag.p, rank.p, n_cand, &na));
    // The internal active list stays the cut tets (the tets the reference's
    // interface accumulators visit); its local-to-global map has -1 for
    // unnumbered vertices.  The reported count is the reference's.
    TF_TRY(ensure(c, c->loc2glo, (size_t)(n_cand > 0 ? 4 * n_cand : 1) + 1));
    if (n_cand > 0) {
        k_legacy_l2g<<<grid_for(c, n_cand), kBlock, 0, c->stream>>>(M, n_cand, c->active.p, c->dof_vert.p, c->loc2glo.p);
        ++c->launches;
    }
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    TF_CUDA(c, cudaGetLastError());
    release(cand);
    release(nonempty);
    release(rank);
    release(flag);
    c->n_active = n_cand;
    c->legacy_n_active = na;
    c->n_dofs = ndofs;
    c->fe = TF_P1IF;
    c->legacy_numbering = true;
    ++c->dof_version;
    return TF_OK;
}

}  // namespace tf
