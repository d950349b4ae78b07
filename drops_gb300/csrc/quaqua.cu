// Isoparametric P2 TraceFEM with the QuaQua mapper (the surfactant.cpp P2
// driver, surfactant/surfactant.cpp:1581-1640).
//
// The discrete surface is the linear interface of the P2 level set's vertex
// values in each cut tet (principal lattice 1), mapped onto the zero level of
// the P2 level set along the recovered gradient:
//   1. the recovered gradient gh (averaging_P2_gradient_recovery,
//      num/gradient_recovery.cpp:30-89): per tet the gradient of the P2 level
//      set at its vertices, the mean of the end values on its edges; every
//      node averages the values of all tets that contain it (running mean in
//      tet order).  k_qq_grad gathers the tets around each node of the
//      interface numbering from the brick structure.
//   2. per quadrature point x0 of the linear interface (Quad5_2D on each
//      facet), the base point: Newton on F(x, s) = (x0 - x - s gh(x), -ls(x))
//      with the Armijo backtracking of newton_solve (num/newton.h:70-113) and
//      the damping bound 0.5 h / |dx| (levelset/levelsetmapper.cpp:289-293).
//      Every iterate is evaluated on the starting tet's own P2 level set and
//      recovered gradient, extended beyond the tet: the reference's
//      locate_new_point (levelsetmapper.cpp:463-490) searches a neighbourhood
//      only while its tet argument is null, and its caller always passes the
//      current tet.
//   3. the Jacobian dp_h = (I + dh Q dn)^-1 Q at the base point
//      (levelsetmapper.cpp:590-638), the surface measure sqrt det Gram(dp_h U)
//      with U an orthonormal basis of the facet (surfactant/ifacetransp.cpp:
//      850-892) and the gradient transformation W = dp_h^T + nl (n / (nl.n) -
//      dp_h nl)^T (ifacetransp.cpp:894-914).
//   4. LocalMassP2CL, LocalLaplaceBeltramiP2CL (W^-1 applied to the tangential
//      P2 gradients) and LocalVectorP2CL (f at the base points)
//      (surfactant/ifacetransp.h:2286-2402).
// The tets are set up once (one thread each); their quadrature points (7 per
// facet, two facets at most on the linear interface) are numbered densely and
// run one thread each, in two passes (the Newton solve; the Jacobian, measure
// and transformation), so that every FP64 warp instruction has 32 active
// lanes.  The element entries are summed per tet over its points in point
// order.
#include <cub/device/device_select.cuh>
#include <thrust/iterator/counting_iterator.h>

#include "tf_internal.cuh"

namespace tf {

namespace {

constexpr int kQqPts = 14;  // quadrature points of a tet, at most

struct Q5 {
    double node[7][3], w[7];
};

struct QqArgs {
    MeshView M;
    const double* ls_vert;
    const double* ls_edge;
    const double* grad;  // recovered gradient per interface DOF (3 per DOF)
    int64_t n_active;
    const int32_t* active;
    const int32_t* loc2glo;
    double* elem_m;  // [n_active][55]
    double* elem_a;  // [n_active][55]
    double* elem_rhs;  // [n_active][10]
    int* status;
    int* newton_max;  // largest Newton iteration count of a point
    double* base;     // [points][8]: base point x, s and its barycentric b (Newton pass -> forms pass)
    Q5 q;
    double tol, armijo, rhs_c;
    int maxiter, max_damping;
};

// one cut tet: vertices, level-set values, barycentric gradients, the
// recovered gradient at its 10 nodes, h, and the linear interface's cut points
struct QqTet {
    double X[4][3], gl[4][3], f[10], gh[10][3], h;
    int cut[4];
    int nr, bnd, npts, pad;
};

// world gradients of the barycentric coordinates (GetTrafoTr) and det J
__device__ void qq_trafo(const double X[4][3], double gl[4][3], double* det) {
    double Mx[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Mx[j][i] = X[i + 1][j] - X[0][j];
    const double d = Mx[0][0] * (Mx[1][1] * Mx[2][2] - Mx[1][2] * Mx[2][1]) -
                     Mx[0][1] * (Mx[1][0] * Mx[2][2] - Mx[1][2] * Mx[2][0]) +
                     Mx[0][2] * (Mx[1][0] * Mx[2][1] - Mx[1][1] * Mx[2][0]);
    double T[3][3];
    T[0][0] = (Mx[1][1] * Mx[2][2] - Mx[1][2] * Mx[2][1]) / d;
    T[0][1] = (Mx[2][0] * Mx[1][2] - Mx[1][0] * Mx[2][2]) / d;
    T[0][2] = (Mx[1][0] * Mx[2][1] - Mx[2][0] * Mx[1][1]) / d;
    T[1][0] = (Mx[2][1] * Mx[0][2] - Mx[0][1] * Mx[2][2]) / d;
    T[1][1] = (Mx[0][0] * Mx[2][2] - Mx[2][0] * Mx[0][2]) / d;
    T[1][2] = (Mx[2][0] * Mx[0][1] - Mx[0][0] * Mx[2][1]) / d;
    T[2][0] = (Mx[0][1] * Mx[1][2] - Mx[1][1] * Mx[0][2]) / d;
    T[2][1] = (Mx[1][0] * Mx[0][2] - Mx[0][0] * Mx[1][2]) / d;
    T[2][2] = (Mx[0][0] * Mx[1][1] - Mx[1][0] * Mx[0][1]) / d;
    const double gref[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 4; ++i)
        for (int r = 0; r < 3; ++r) gl[i][r] = T[r][0] * gref[i][0] + T[r][1] * gref[i][1] + T[r][2] * gref[i][2];
    *det = d;
}

__device__ void qq_tet_data(const MeshView& M, const double* lsv, const double* lse, int64_t t, double X[4][3],
                            double f[10], int32_t tv[4], int32_t te[6]) {
    mesh_tet(M, t, tv, te);
    for (int k = 0; k < 4; ++k) {
        mesh_coord(M, tv[k], X[k]);
        f[k] = lsv[tv[k]];
    }
    for (int k = 0; k < 6; ++k) f[4 + k] = lse[te[k]];
}

// gradient of the tet's P2 function f at its local vertex k
__device__ void qq_vertex_grad(const double gl[4][3], const double f[10], int k, double g[3]) {
    for (int r = 0; r < 3; ++r) {
        double s = 0.;
        for (int j = 0; j < 4; ++j) s += f[j] * ((j == k ? 3. : -1.) * gl[j][r]);
        for (int e = 0; e < 6; ++e) {
            const int a = ev0(e), b = ev1(e);
            s += f[4 + e] * (4. * ((b == k ? 1. : 0.) * gl[a][r] + (a == k ? 1. : 0.) * gl[b][r]));
        }
        g[r] = s;
    }
}

// the recovered gradient at every node that carries an interface DOF: the
// running mean over the node's tets in tet order.  On the uniform Kuhn brick
// the barycentric gradients of a tet depend only on its type (its index in the
// cube) up to the rounding of the vertex coordinates (~1e-14 relative), so the
// block forms them once per type; the running mean's weights (n-1)/n and 1/n
// come from a table of the same FP64 divisions.
constexpr int kQqMaxTets = 48;  // tets around a node (24 on the Kuhn brick)
// the nodes (vertex, or nv + edge) that carry an interface DOF, in node order
struct QqHasDof {
    int64_t nv;
    const int32_t* dof_vert;
    const int32_t* dof_edge;
    __device__ bool operator()(int32_t node) const {
        return (node < nv ? dof_vert[node] : dof_edge[node - nv]) >= 0;
    }
};

// one thread per interface DOF, the DOFs in node order: the nodes without one
// do no work and a warp holds vertices or edges, whose gathers differ (up to
// 48 candidate tets around a vertex, fewer around an edge), so that the FP64
// work of the gradients runs in full warps
__global__ void k_qq_grad(MeshView M, const double* __restrict__ lsv, const double* __restrict__ lse,
                          const int32_t* __restrict__ dof_vert, const int32_t* __restrict__ dof_edge,
                          const int32_t* __restrict__ nodes, int64_t m, double* __restrict__ grad) {
    __shared__ double glT[6][4][3];
    __shared__ double rmA[kQqMaxTets + 1], rmB[kQqMaxTets + 1];
    const Brick& B = M.b;
    if (threadIdx.x < 6) {
        double X[4][3], f[10], gl[4][3], det;
        int32_t tv[4], te[6];
        qq_tet_data(M, lsv, lse, threadIdx.x, X, f, tv, te);
        qq_trafo(X, gl, &det);
        for (int k = 0; k < 4; ++k)
            for (int r = 0; r < 3; ++r) glT[threadIdx.x][k][r] = gl[k][r];
    }
    for (int k = threadIdx.x; k <= kQqMaxTets; k += blockDim.x) {
        const double n = (double)(k > 0 ? k : 1);
        rmA[k] = (n - 1.) / n;
        rmB[k] = 1. / n;
    }
    __syncthreads();
    const int64_t nvert = M.nv;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t node = nodes[i];
        const bool isv = node < nvert;
        const int64_t id = isv ? node : node - nvert;
        const int32_t dof = isv ? dof_vert[id] : dof_edge[id];
        // lower vertex (i3, i2, i1) of the node
        int64_t v = id;
        int d3 = 0, d2 = 0, d1 = 0;
        if (!isv) {
            int cls = 0;
            while (cls < 6 && id >= B.eoff[cls + 1]) ++cls;
            const int code = (int)((0x7653421 >> (4 * cls)) & 0xf);  // class -> (d3 d2 d1) bits: 1,2,4,3,5,6,7
            d3 = (code >> 2) & 1;
            d2 = (code >> 1) & 1;
            d1 = code & 1;
            const int64_t r = id - B.eoff[cls];
            const int64_t w1 = B.n1 + 1 - d1, w2 = B.n2 + 1 - d2;
            const int64_t a1 = r % w1, q = r / w1, a2 = q % w2, a3 = q / w2;
            v = (a3 * (B.n2 + 1) + a2) * (B.n1 + 1) + a1;
        }
        const int64_t i1 = v % (B.n1 + 1), q = v / (B.n1 + 1), i2 = q % (B.n2 + 1), i3 = q / (B.n2 + 1);
        double avg[3] = {0., 0., 0.};
        int n = 0;
        for (int a3 = 1; a3 >= 0; --a3)
            for (int a2 = 1; a2 >= 0; --a2)
                for (int a1 = 1; a1 >= 0; --a1) {
                    const int64_t c3 = i3 - a3, c2 = i2 - a2, c1 = i1 - a1;
                    if (c3 < 0 || c2 < 0 || c1 < 0 || c3 >= B.n3 || c2 >= B.n2 || c1 >= B.n1) continue;
                    if (a3 + d3 > 1 || a2 + d2 > 1 || a1 + d1 > 1) continue;
                    const int64_t cube = (c3 * B.n2 + c2) * B.n1 + c1;
                    for (int l = 0; l < 6; ++l) {
                        const int64_t t = 6 * cube + l;
                        double f[10], gl[4][3];
                        int32_t tv[4], te[6];
                        brick_tet(B, t, 0, 0, tv, te);
                        int k = -1;
                        if (isv) {
                            for (int j = 0; j < 4; ++j)
                                if (tv[j] == (int32_t)id) k = j;
                        } else {
                            for (int j = 0; j < 6; ++j)
                                if (te[j] == (int32_t)id) k = 4 + j;
                        }
                        if (k < 0) continue;
                        for (int j = 0; j < 4; ++j) f[j] = lsv[tv[j]];
                        for (int j = 0; j < 6; ++j) f[4 + j] = lse[te[j]];
                        for (int j = 0; j < 4; ++j)
                            for (int r = 0; r < 3; ++r) gl[j][r] = glT[l][j][r];
                        double val[3];
                        if (k < 4) {
                            qq_vertex_grad(gl, f, k, val);
                        } else {
                            double ga[3], gb[3];
                            qq_vertex_grad(gl, f, ev0(k - 4), ga);
                            qq_vertex_grad(gl, f, ev1(k - 4), gb);
                            for (int r = 0; r < 3; ++r) val[r] = 0.5 * (ga[r] + gb[r]);
                        }
                        n = n < kQqMaxTets ? n + 1 : n;
                        for (int r = 0; r < 3; ++r) avg[r] = rmA[n] * avg[r] + rmB[n] * val[r];
                    }
                }
        for (int r = 0; r < 3; ++r) grad[3 * (int64_t)dof + r] = avg[r];
    }
}

// P2 values and world gradients at barycentric b (FE_P2CL)
__device__ void qq_p2(const double b[4], const double gl[4][3], double phi[10], double g[10][3]) {
    for (int i = 0; i < 4; ++i) {
        phi[i] = b[i] * (2. * b[i] - 1.);
        for (int r = 0; r < 3; ++r) g[i][r] = (4. * b[i] - 1.) * gl[i][r];
    }
    for (int e = 0; e < 6; ++e) {
        const int a = ev0(e), c = ev1(e);
        phi[4 + e] = 4. * b[a] * b[c];
        for (int r = 0; r < 3; ++r) g[4 + e][r] = 4. * (b[c] * gl[a][r] + b[a] * gl[c][r]);
    }
}

// ls, its gradient, gh and (optionally) dgh = sum_k gh_k (x) grad phi_k of the tet's polynomials at b;
// the basis functions one at a time (FE_P2CL's values and gradients), every sum in k order
__device__ void qq_eval(const QqTet& S, const double b[4], double* ls, double gls[3], double gh[3], double (*dgh)[3]) {
    double l = 0., s[3] = {0., 0., 0.}, s2[3] = {0., 0., 0.}, v[3][3] = {{0., 0., 0.}, {0., 0., 0.}, {0., 0., 0.}};
#pragma unroll 1
    for (int k = 0; k < 10; ++k) {
        double phi, g[3];
        if (k < 4) {
            phi = b[k] * (2. * b[k] - 1.);
            for (int r = 0; r < 3; ++r) g[r] = (4. * b[k] - 1.) * S.gl[k][r];
        } else {
            const int a = ev0(k - 4), c = ev1(k - 4);
            phi = 4. * b[a] * b[c];
            for (int r = 0; r < 3; ++r) g[r] = 4. * (b[c] * S.gl[a][r] + b[a] * S.gl[c][r]);
        }
        l += S.f[k] * phi;
        for (int r = 0; r < 3; ++r) {
            s[r] += S.f[k] * g[r];
            s2[r] += S.gh[k][r] * phi;
        }
        if (dgh)
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) v[r][c] += S.gh[k][r] * g[c];
    }
    *ls = l;
    for (int r = 0; r < 3; ++r) {
        gls[r] = s[r];
        gh[r] = s2[r];
    }
    if (dgh)
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) dgh[r][c] = v[r][c];
}

__device__ void qq_w2b(const QqTet& S, const double x[3], double b[4]) {
    const double d[3] = {x[0] - S.X[0][0], x[1] - S.X[0][1], x[2] - S.X[0][2]};
    b[0] = 1.;
    for (int k = 1; k < 4; ++k) {
        b[k] = S.gl[k][0] * d[0] + S.gl[k][1] * d[1] + S.gl[k][2] * d[2];
        b[0] -= b[k];
    }
}

// Gaussian elimination with partial pivoting, n <= 4; false on a zero pivot
__device__ bool qq_solve(int n, double A[4][4], double x[4]) {
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i)
            if (fabs(A[i][k]) > fabs(A[p][k])) p = i;
        if (A[p][k] == 0.) return false;
        if (p != k) {
            for (int j = 0; j < n; ++j) {
                const double t = A[k][j];
                A[k][j] = A[p][j];
                A[p][j] = t;
            }
            const double t = x[k];
            x[k] = x[p];
            x[p] = t;
        }
        for (int i = k + 1; i < n; ++i) {
            const double mlt = A[i][k] / A[k][k];
            for (int j = k; j < n; ++j) A[i][j] -= mlt * A[k][j];
            x[i] -= mlt * x[k];
        }
    }
    for (int k = n - 1; k >= 0; --k) {
        double s = x[k];
        for (int j = k + 1; j < n; ++j) s -= A[k][j] * x[j];
        x[k] = s / A[k][k];
    }
    return true;
}

__device__ inline double nrm3(const double v[3]) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
__device__ inline double dt3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// The tets' data (coordinates, level set, barycentric gradients, the
// recovered gradient at the 10 nodes, the linear interface's cut points) are
// set up once per tet; the quadrature points of all tets are then numbered
// densely (7 per facet, a scan over the tets) and run one thread each: the
// Newton solve for the base point, then the mapping's Jacobian, the measure
// and the gradient transformation (FP64 work: full warps keep all 32 lanes of
// every FP64 warp instruction busy, where a half-warp per tet used 7 or 14).
// The element entries are summed per tet over its points in point order.
constexpr int kQqPtData = 42;  // per point: w |det|, f(y), the 10 P2 values, the 10 transformed surface gradients

__global__ void k_qq_tets(QqArgs a, QqTet* __restrict__ tets, int32_t* __restrict__ npts) {
    for (int64_t qa = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; qa < a.n_active;
         qa += (int64_t)gridDim.x * blockDim.x) {
        QqTet& S = tets[qa];
        const int64_t t = a.active[qa];
        int32_t tv[4], te[6];
        qq_tet_data(a.M, a.ls_vert, a.ls_edge, t, S.X, S.f, tv, te);
        double det;
        qq_trafo(S.X, S.gl, &det);
        S.h = cbrt(fabs(det));
        for (int q = 0; q < 30; ++q) {
            const int k = q / 3, r = q - 3 * k;
            S.gh[k][r] = a.grad[3 * (int64_t)a.loc2glo[qa * 10 + k] + r];
        }
        // the linear interface of the vertex values (SignTraitsCL / RefPatchCL on one sub-tet)
        int sg[4], nz = 0;
        bool mixed = false;
        for (int k = 0; k < 4; ++k) {
            sg[k] = (S.f[k] > 0.) - (S.f[k] < 0.);
            mixed |= sg[k] != sg[0];
            nz += sg[k] == 0;
        }
        int nr = 0;
        for (int k = 0; k < 4; ++k) S.cut[k] = 0;
        if (mixed) {
            for (int k = 0; k < 4; ++k)
                if (sg[k] == 0) S.cut[nr++] = k;
            for (int e = 0; e < 6 && nr < 4; ++e)
                if (sg[ev0(e)] * sg[ev1(e)] == -1) S.cut[nr++] = e + 4;
        }
        if (nz == 4) atomicCAS(a.status, 0, TF_ERR_ZERO_PATTERN);
        const int nf = nr >= 3 ? nr - 2 : 0;
        S.nr = nr;
        S.bnd = nz == 3;
        S.npts = 7 * nf;
        npts[qa] = 7 * nf;
    }
}

__global__ void k_qq_point_tets(int64_t na, const int32_t* __restrict__ npts, const int32_t* __restrict__ off,
                                int32_t* __restrict__ pt_tet) {
    for (int64_t qa = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; qa < na; qa += (int64_t)gridDim.x * blockDim.x)
        for (int j = 0; j < npts[qa]; ++j) pt_tet[off[qa] + j] = (int32_t)qa;
}

// PH 0: the base point (x, s) by Newton and its barycentric b; PH 1: from the
// stored base point, the point's weight x measure, f(y), P2 values and
// transformed surface gradients.  Both phases rebuild the facet geometry of
// the point with the same operations.
template <int PH>
__global__ void __launch_bounds__(128) k_qq_points(QqArgs a, const QqTet* __restrict__ tets,
                                                   const int32_t* __restrict__ off,
                                                   const int32_t* __restrict__ pt_tet, int64_t npt,
                                                   double* __restrict__ pdata) {
    for (int64_t pid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pid < npt;
         pid += (int64_t)gridDim.x * blockDim.x) {
        const int32_t qa = pt_tet[pid];
        const QqTet& S = tets[qa];
        const int lane = (int)(pid - off[qa]);
        const int* cut = S.cut;
        const bool bnd = S.bnd != 0;
        auto fvert = [&](int f, int j, double b[4]) {
            const int cv = cut[f + j];
            for (int c = 0; c < 4; ++c) b[c] = 0.;
            if (cv < 4) {
                b[cv] = 1.;
            } else {
                const int p = ev0(cv - 4), s = ev1(cv - 4);
                const double tt = S.f[p] / (S.f[p] - S.f[s]);
                b[p] = 1.0 - tt;
                b[s] = tt;
            }
        };
        auto world = [&](const double b[4], double x[3]) {
            for (int r = 0; r < 3; ++r) x[r] = S.X[0][r] * b[0] + S.X[1][r] * b[1] + S.X[2][r] * b[2] + S.X[3][r] * b[3];
        };
        {
            const int f = lane / 7, qn = lane - 7 * f;
            double B[3][4], W3[3][3];
            for (int j = 0; j < 3; ++j) {
                fvert(f, j, B[j]);
                world(B[j], W3[j]);
            }
            double u[3], v[3], cr[3];
            for (int r = 0; r < 3; ++r) {
                u[r] = W3[1][r] - W3[0][r];
                v[r] = W3[2][r] - W3[0][r];
            }
            cr[0] = u[1] * v[2] - u[2] * v[1];
            cr[1] = u[2] * v[0] - u[0] * v[2];
            cr[2] = u[0] * v[1] - u[1] * v[0];
            const double fdet = nrm3(cr) * (bnd ? 0.5 : 1.0);
            // normal of facet 0 (the facets of the linear interface are coplanar)
            double nl[3];
            {
                double B0[3][4], P0[3][3], u0[3], v0[3];
                for (int j = 0; j < 3; ++j) {
                    fvert(0, j, B0[j]);
                    world(B0[j], P0[j]);
                }
                for (int r = 0; r < 3; ++r) {
                    u0[r] = P0[1][r] - P0[0][r];
                    v0[r] = P0[2][r] - P0[0][r];
                }
                nl[0] = u0[1] * v0[2] - u0[2] * v0[1];
                nl[1] = u0[2] * v0[0] - u0[0] * v0[2];
                nl[2] = u0[0] * v0[1] - u0[1] * v0[0];
                const double nn = nrm3(nl);
                for (int r = 0; r < 3; ++r) nl[r] /= nn;
            }
            // orthonormal basis of the facet plane
            double U0[3], U1[3];
            const double nu = nrm3(u);
            for (int r = 0; r < 3; ++r) U0[r] = u[r] / nu;
            const double vu = dt3(v, U0);
            for (int r = 0; r < 3; ++r) U1[r] = v[r] - vu * U0[r];
            const double nv = nrm3(U1);
            for (int r = 0; r < 3; ++r) U1[r] /= nv;
            double bq[4];
            for (int c = 0; c < 4; ++c) bq[c] = B[0][c] * a.q.node[qn][0] + B[1][c] * a.q.node[qn][1] + B[2][c] * a.q.node[qn][2];
            const double wq = fdet * a.q.w[qn];
            double* const bp = a.base + (size_t)pid * 8;
            double x[4], b[4];
            double ls, gls[3], gh[3], dgh[3][3];
            if constexpr (PH == 0) {
            // Newton for the base point on the tet's extended polynomials
            double x0[3];
            world(bq, x0);
            for (int i = 0; i < 3; ++i) x[i] = x0[i];
            x[3] = 0.;
            for (int i = 0; i < 4; ++i) b[i] = bq[i];
            double F[4];
            qq_eval(S, b, &ls, gls, gh, nullptr);
            F[0] = F[1] = F[2] = 0.;
            F[3] = -ls;
            int iter;
            for (iter = 0;; ++iter) {
                const double normF = sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3]);
                if (iter >= a.maxiter || normF < a.tol) break;
                qq_eval(S, b, &ls, gls, gh, dgh);
                double dF[4][4], A4[4][4], dx[4];
                for (int i = 0; i < 3; ++i) {
                    for (int j = 0; j < 3; ++j) dF[i][j] = -x[3] * dgh[i][j];
                    dF[i][i] -= 1.;
                    dF[i][3] = -gh[i];
                    dF[3][i] = -gls[i];
                }
                dF[3][3] = 0.;
                for (int i = 0; i < 4; ++i) {
                    dx[i] = F[i];
                    for (int j = 0; j < 4; ++j) A4[i][j] = dF[i][j];
                }
                if (!qq_solve(4, A4, dx)) {
                    atomicCAS(a.status, 0, TF_ERR_BAD_INPUT);
                    break;
                }
                double Jd[4] = {0., 0., 0., 0.};
                for (int i = 0; i < 4; ++i)
                    for (int j = 0; j < 4; ++j) Jd[i] += dF[i][j] * dx[j];
                const double slope = a.armijo * (F[0] * Jd[0] + F[1] * Jd[1] + F[2] * Jd[2] + F[3] * Jd[3]) / normF;
                double l = 0.5 * S.h / sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
                if (!(l < 1.)) l = 1.;
                double bn[4], Fn[4];
                bool accepted = false;
                for (int j = 0; j < a.max_damping && l >= 1e-7; ++j, l *= 0.5) {
                    double xn[4];
                    for (int i = 0; i < 4; ++i) xn[i] = x[i] - l * dx[i];
                    qq_w2b(S, xn, bn);
                    double lsn, gn[3], ghn[3];
                    qq_eval(S, bn, &lsn, gn, ghn, nullptr);
                    for (int i = 0; i < 3; ++i) Fn[i] = x0[i] - xn[i] - xn[3] * ghn[i];
                    Fn[3] = -lsn;
                    if (sqrt(Fn[0] * Fn[0] + Fn[1] * Fn[1] + Fn[2] * Fn[2] + Fn[3] * Fn[3]) < normF + slope * l) {
                        accepted = true;
                        break;
                    }
                }
                if (l < 1e-7) break;
                for (int i = 0; i < 4; ++i) x[i] -= l * dx[i];
                if (!accepted) {  // newton_solve takes the last halved factor without evaluating it
                    qq_w2b(S, x, bn);
                    double lsn, gn[3], ghn[3];
                    qq_eval(S, bn, &lsn, gn, ghn, nullptr);
                    for (int i = 0; i < 3; ++i) Fn[i] = x0[i] - x[i] - x[3] * ghn[i];
                    Fn[3] = -lsn;
                }
                for (int i = 0; i < 4; ++i) {
                    b[i] = bn[i];
                    F[i] = Fn[i];
                }
            }
            atomicMax(a.newton_max, iter);
            for (int i = 0; i < 4; ++i) {
                bp[i] = x[i];
                bp[4 + i] = b[i];
            }
            } else {
            double* const P = pdata + (size_t)pid * kQqPtData;
            for (int i = 0; i < 4; ++i) {
                x[i] = bp[i];
                b[i] = bp[4 + i];
            }
            // Jacobian of the mapping at the base point
            qq_eval(S, b, &ls, gls, gh, dgh);
            const double ngh = nrm3(gh), dh = x[3] * ngh, ngl = nrm3(gls);
            double qv[3], n[3], tq[3];
            for (int r = 0; r < 3; ++r) {
                qv[r] = gh[r] / ngh;
                n[r] = gls[r] / ngl;
            }
            for (int c = 0; c < 3; ++c) tq[c] = dgh[0][c] * qv[0] + dgh[1][c] * qv[1] + dgh[2][c] * qv[2];
            const double qdn = dt3(qv, n);
            double dn[3][3], Q[3][3], Bm[3][3], dph[3][3];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) {
                    dn[r][c] = (1. / ngh) * (dgh[r][c] - qv[r] * tq[c]);
                    Q[r][c] = (r == c ? 1. : 0.) - (qv[r] / qdn) * n[c];
                }
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) {
                    double s = 0.;
                    for (int k = 0; k < 3; ++k) s += Q[r][k] * dn[k][c];
                    Bm[r][c] = (r == c ? 1. : 0.) + dh * s;
                }
            for (int col = 0; col < 3; ++col) {
                double A4[4][4], rhs[4] = {Q[0][col], Q[1][col], Q[2][col], 0.};
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) A4[r][c] = Bm[r][c];
                qq_solve(3, A4, rhs);
                for (int r = 0; r < 3; ++r) dph[r][col] = rhs[r];
            }
            // surface measure and the gradient transformation
            double DU0[3], DU1[3], dnl[3];
            for (int r = 0; r < 3; ++r) {
                DU0[r] = dph[r][0] * U0[0] + dph[r][1] * U0[1] + dph[r][2] * U0[2];
                DU1[r] = dph[r][0] * U1[0] + dph[r][1] * U1[1] + dph[r][2] * U1[2];
                dnl[r] = dph[r][0] * nl[0] + dph[r][1] * nl[1] + dph[r][2] * nl[2];
            }
            const double g00 = dt3(DU0, DU0), g01 = dt3(DU0, DU1), g11 = dt3(DU1, DU1);
            const double absd = sqrt(g00 * g11 - g01 * g01);
            const double nln = dt3(nl, n);
            double Wi[3][3];
            for (int col = 0; col < 3; ++col) {
                double A4[4][4], rhs[4] = {col == 0 ? 1. : 0., col == 1 ? 1. : 0., col == 2 ? 1. : 0., 0.};
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) A4[r][c] = dph[c][r] + nl[r] * (n[c] / nln - dnl[c]);
                qq_solve(3, A4, rhs);
                for (int r = 0; r < 3; ++r) Wi[r][col] = rhs[r];
            }
            double phi[10], g[10][3];
            qq_p2(bq, S.gl, phi, g);
            P[0] = wq * absd;
            double y[3];
            for (int r = 0; r < 3; ++r) y[r] = x[r];
            P[1] = a.rhs_c * y[0] * y[1] * y[2];
            for (int i = 0; i < 10; ++i) {
                P[2 + i] = phi[i];
                const double gn = dt3(g[i], nl);
                double tg[3];
                for (int r = 0; r < 3; ++r) tg[r] = g[i][r] - gn * nl[r];
                for (int r = 0; r < 3; ++r) P[12 + 3 * i + r] = Wi[r][0] * tg[0] + Wi[r][1] * tg[1] + Wi[r][2] * tg[2];
            }
            }
        }
    }
}

// the element entries of tet qa, summed over its points in point order: 55 M, 55 A, 10 b; one warp per
// tet, its points' records staged in shared memory
constexpr int kQqSumWarps = 4;
__global__ void __launch_bounds__(32 * kQqSumWarps) k_qq_sums(QqArgs a, const int32_t* __restrict__ off,
                                                             const double* __restrict__ pdata) {
    __shared__ double rec[kQqSumWarps][kQqPts * kQqPtData];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double* R = rec[w];
    for (int64_t qa = blockIdx.x * (int64_t)kQqSumWarps + w; qa < a.n_active; qa += (int64_t)gridDim.x * kQqSumWarps) {
        const int64_t p0 = off[qa];
        const int npts = off[qa + 1] - off[qa];
        for (int k = lane; k < npts * kQqPtData; k += 32) R[k] = pdata[(size_t)p0 * kQqPtData + k];
        __syncwarp();
        for (int e = lane; e < 120; e += 32) {
            double s = 0.;
            if (e < 110) {
                const int k = e < 55 ? e : e - 55;
                int i = 0, rem = k;
                while (rem >= 10 - i) {
                    rem -= 10 - i;
                    ++i;
                }
                const int j = i + rem;
                for (int p = 0; p < npts; ++p) {
                    const double* P = R + p * kQqPtData;
                    if (e < 55)
                        s += P[0] * P[2 + i] * P[2 + j];
                    else
                        s += P[0] * dt3(P + 12 + 3 * i, P + 12 + 3 * j);
                }
                (e < 55 ? a.elem_m : a.elem_a)[qa * 55 + k] = s;
            } else {
                const int i = e - 110;
                for (int p = 0; p < npts; ++p) {
                    const double* P = R + p * kQqPtData;
                    s += P[0] * P[1] * P[2 + i];
                }
                a.elem_rhs[qa * 10 + i] = s;
            }
        }
        __syncwarp();
    }
}

}  // namespace

int quaqua_elements(Context* c, double rhs_c, double tol, int maxiter, int* newton_max) {
    if (c->mesh.explicit_mesh || c->mesh.nbatch)
        return set_err(c, TF_ERR_BAD_INPUT, "quaqua: needs a single brick mesh");
    if (c->fe != TF_P2IF || c->legacy_numbering)
        return set_err(c, TF_ERR_BAD_INPUT, "quaqua: needs the P2IF numbering of DistributeDOFs");
    const int64_t na = c->n_active, m = c->n_dofs;
    TF_TRY(ensure(c, c->qq_grad, (size_t)(3 * (m > 0 ? m : 1))));
    TF_TRY(ensure(c, c->elem, (size_t)TF_NUM_FORMS * (size_t)(na > 0 ? na : 1) * 55));
    TF_TRY(ensure(c, c->elem_rhs, (size_t)(na > 0 ? na : 1) * 10));
    // per tet its data; per point (at most 14 per tet) the base point and the point data; the index buffer
    // first holds the DOFs' nodes, then the points per tet, their offsets and each point's tet
    const size_t tet_words = ((size_t)(na > 0 ? na : 1) * sizeof(QqTet) + 7) / 8;
    const size_t max_pts = (size_t)(na > 0 ? na : 1) * kQqPts;
    TF_TRY(ensure(c, c->qq_base, tet_words + max_pts * (8 + kQqPtData)));
    TF_TRY(ensure(c, c->qq_idx, std::max((size_t)(2 * (na + 1)) + max_pts, (size_t)(m > 0 ? m : 1) + 1)));
    QqTet* tets = reinterpret_cast<QqTet*>(c->qq_base.p);
    double* pdata = c->qq_base.p + tet_words + max_pts * 8;
    int32_t* npts = c->qq_idx.p;
    int32_t* off = npts + (na + 1);
    int32_t* pt_tet = off + (na + 1);
    const int64_t nnodes = c->mesh.nv + c->mesh.ne;
    if (nnodes > INT32_MAX) return set_err(c, TF_ERR_CAPACITY, "quaqua: 32-bit node ids");
    {
        const QqHasDof pred{c->mesh.nv, c->dof_vert.p, c->dof_edge.p};
        thrust::counting_iterator<int32_t> first(0);
        size_t bytes = 0;
        TF_CUDA(c, cub::DeviceSelect::If(nullptr, bytes, first, c->qq_idx.p, c->qq_idx.p + m, (int)nnodes, pred,
                                         c->stream));
        TF_TRY(ensure(c, c->order_tmp, bytes > 0 ? bytes : 1));
        TF_CUDA(c, cub::DeviceSelect::If(c->order_tmp.p, bytes, first, c->qq_idx.p, c->qq_idx.p + m, (int)nnodes, pred,
                                         c->stream));
    }
    k_qq_grad<<<grid_for(c, m), kBlock, 0, c->stream>>>(c->mesh, c->ls_vert.p, c->ls_edge.p, c->dof_vert.p,
                                                        c->dof_edge.p, c->qq_idx.p, m, c->qq_grad.p);
    c->launches += 3;  // with the selection's
    TF_CUDA(c, cudaGetLastError());
    QqArgs a{};
    a.M = c->mesh;
    a.ls_vert = c->ls_vert.p;
    a.ls_edge = c->ls_edge.p;
    a.grad = c->qq_grad.p;
    a.n_active = na;
    a.active = c->active.p;
    a.loc2glo = c->loc2glo.p;
    a.elem_m = c->elem.p + (size_t)TF_FORM_M * na * 55;
    a.elem_a = c->elem.p + (size_t)TF_FORM_A * na * 55;
    a.elem_rhs = c->elem_rhs.p;
    a.status = c->status.p;
    a.newton_max = c->status.p + 3;
    a.base = c->qq_base.p + tet_words;
    const double s15 = std::sqrt(15.0);
    const double A1 = (6.0 - s15) / 21.0, B1 = (9.0 + 2.0 * s15) / 21.0;
    const double A2 = (6.0 + s15) / 21.0, B2 = (9.0 - 2.0 * s15) / 21.0;
    const double nodes7[7][3] = {{1. / 3., 1. / 3., 1. / 3.}, {A1, A1, B1}, {A1, B1, A1}, {B1, A1, A1},
                                 {A2, A2, B2}, {A2, B2, A2}, {B2, A2, A2}};
    for (int i = 0; i < 7; ++i)
        for (int j = 0; j < 3; ++j) a.q.node[i][j] = nodes7[i][j];
    a.q.w[0] = 9. / 80.;
    for (int i = 1; i <= 3; ++i) a.q.w[i] = (155. - s15) / 2400.;
    for (int i = 4; i <= 6; ++i) a.q.w[i] = (155. + s15) / 2400.;
    a.tol = tol;
    a.armijo = 1e-4;
    a.rhs_c = rhs_c;
    a.maxiter = maxiter;
    a.max_damping = 8;
    TF_CUDA(c, cudaMemsetAsync(c->status.p, 0, 4 * sizeof(int), c->stream));
    if (na > 0) {
        TimedLaunch tl(c, TF_K_ASSEMBLE);
        k_qq_tets<<<grid_for(c, na), kBlock, 0, c->stream>>>(a, tets, npts);
        TF_CUDA(c, cudaGetLastError());
        int64_t npt = 0;
        TF_TRY(exclusive_scan_i32_to_i32(c, npts, off, na, &npt));  // off[na] = npt
        if (npt > (int64_t)max_pts) return set_err(c, TF_ERR_INTERNAL, "quaqua: point count");
        k_qq_point_tets<<<grid_for(c, na), kBlock, 0, c->stream>>>(na, npts, off, pt_tet);
        const int gp = grid_for(c, npt, 128);
        k_qq_points<0><<<gp, 128, 0, c->stream>>>(a, tets, off, pt_tet, npt, pdata);
        k_qq_points<1><<<gp, 128, 0, c->stream>>>(a, tets, off, pt_tet, npt, pdata);
        k_qq_sums<<<grid_for(c, (na + kQqSumWarps - 1) / kQqSumWarps, 1, 8), 32 * kQqSumWarps, 0, c->stream>>>(
            a, off, pdata);
        c->launches += 6;  // with the scan's
        TF_CUDA(c, cudaGetLastError());
    }
    int h[4] = {0, 0, 0, 0};
    TF_CUDA(c, cudaMemcpyAsync(h, c->status.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    TF_CUDA(c, cudaStreamSynchronize(c->stream));
    if (h[0] == TF_ERR_ZERO_PATTERN)
        return set_err(c, h[0], "quaqua: a tet with a zero level set at all four vertices");
    if (h[0]) return set_err(c, h[0], "quaqua: singular Newton system");
    if (newton_max) *newton_max = h[3];
    return TF_OK;
}

}  // namespace tf
