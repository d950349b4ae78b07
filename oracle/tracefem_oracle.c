/*
 * CPU oracle for the TraceFEM hot path of DROPS -- TEST INFRASTRUCTURE ONLY.
 * See tracefem_oracle.h.  Compile with -ffp-contract=off so that x86 and Arm
 * builds round identically.
 */
#include "tracefem_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;
void orc_set_threads(int n) { g_threads = n; }

/* local edge -> local vertices (geom/topo.cpp VertOfEdgeAr, first 6 rows) */
static const int EV[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};

/* ======================================================================= */
/* mesh                                                                      */
/* ======================================================================= */
/* The 7 edge directions of the Kuhn brick, as offsets (d3, d2, d1).       */
static const int EDIR[7][3] = {{0, 0, 1}, {0, 1, 0}, {1, 0, 0}, {0, 1, 1}, {1, 0, 1}, {1, 1, 0}, {1, 1, 1}};

int64_t orc_brick_num_vertices(int n1, int n2, int n3) { return (int64_t)(n1 + 1) * (n2 + 1) * (n3 + 1); }
int64_t orc_brick_num_tets(int n1, int n2, int n3) { return (int64_t)6 * n1 * n2 * n3; }
static int64_t edir_count(int t, int n1, int n2, int n3) {
    return (int64_t)(n3 + 1 - EDIR[t][0]) * (n2 + 1 - EDIR[t][1]) * (n1 + 1 - EDIR[t][2]);
}
int64_t orc_brick_num_edges(int n1, int n2, int n3) {
    int64_t s = 0;
    for (int t = 0; t < 7; ++t) s += edir_count(t, n1, n2, n3);
    return s;
}

/* Kuhn split of one cube into 6 tets, local vertex offsets (i3,i2,i1) in the
 * order of BrickBuilderCL::build_ser_impl (geom/builder.cpp:151-176).      */
static const int KUHN[6][4][3] = {
    {{0, 0, 0}, {0, 0, 1}, {0, 1, 1}, {1, 1, 1}}, {{0, 0, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}},
    {{0, 0, 0}, {0, 1, 0}, {0, 1, 1}, {1, 1, 1}}, {{0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 1, 1}},
    {{0, 0, 0}, {1, 0, 0}, {1, 0, 1}, {1, 1, 1}}, {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {1, 1, 1}}};

void orc_brick(const double orig[3], const double e1[3], const double e2[3], const double e3[3], int n1,
               int n2, int n3, double* coords, int32_t* tet_v, int32_t* tet_e, int32_t* edge_v) {
    double o1[3], o2[3], o3[3];
    for (int c = 0; c < 3; ++c) {
        o1[c] = (1.0 / (double)n1) * e1[c];
        o2[c] = (1.0 / (double)n2) * e2[c];
        o3[c] = (1.0 / (double)n3) * e3[c];
    }
    int64_t v = 0;
    for (int i3 = 0; i3 <= n3; ++i3)
        for (int i2 = 0; i2 <= n2; ++i2)
            for (int i1 = 0; i1 <= n1; ++i1, ++v)
                for (int c = 0; c < 3; ++c)
                    coords[3 * v + c] = ((orig[c] + (double)i1 * o1[c]) + (double)i2 * o2[c]) + (double)i3 * o3[c];
    int64_t eoff[8];
    eoff[0] = 0;
    for (int t = 0; t < 7; ++t) eoff[t + 1] = eoff[t] + edir_count(t, n1, n2, n3);
    if (edge_v) {
        for (int t = 0; t < 7; ++t) {
            int64_t k = eoff[t];
            for (int i3 = 0; i3 <= n3 - EDIR[t][0]; ++i3)
                for (int i2 = 0; i2 <= n2 - EDIR[t][1]; ++i2)
                    for (int i1 = 0; i1 <= n1 - EDIR[t][2]; ++i1, ++k) {
                        int64_t a = ((int64_t)i3 * (n2 + 1) + i2) * (n1 + 1) + i1;
                        int64_t b = ((int64_t)(i3 + EDIR[t][0]) * (n2 + 1) + i2 + EDIR[t][1]) * (n1 + 1) + i1 + EDIR[t][2];
                        edge_v[2 * k] = (int32_t)a;
                        edge_v[2 * k + 1] = (int32_t)b;
                    }
        }
    }
    int64_t tt = 0;
    for (int i3 = 0; i3 < n3; ++i3)
        for (int i2 = 0; i2 < n2; ++i2)
            for (int i1 = 0; i1 < n1; ++i1)
                for (int l = 0; l < 6; ++l, ++tt) {
                    int p[4][3];
                    for (int k = 0; k < 4; ++k) {
                        p[k][0] = i3 + KUHN[l][k][0];
                        p[k][1] = i2 + KUHN[l][k][1];
                        p[k][2] = i1 + KUHN[l][k][2];
                        tet_v[4 * tt + k] = (int32_t)(((int64_t)p[k][0] * (n2 + 1) + p[k][1]) * (n1 + 1) + p[k][2]);
                    }
                    if (tet_e) {
                        for (int k = 0; k < 6; ++k) {
                            const int* a = p[EV[k][0]];
                            const int* b = p[EV[k][1]];
                            int d[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
                            int t;
                            for (t = 0; t < 7; ++t)
                                if (EDIR[t][0] == d[0] && EDIR[t][1] == d[1] && EDIR[t][2] == d[2]) break;
                            int64_t idx = eoff[t] + ((int64_t)a[0] * (n2 + 1 - EDIR[t][1]) + a[1]) * (n1 + 1 - EDIR[t][2]) + a[2];
                            tet_e[6 * tt + k] = (int32_t)idx;
                        }
                    }
                }
}

/* ======================================================================= */
/* level sets                                                                */
/* ======================================================================= */
static double norm3(const double x[3]) { return sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]); }

double orc_ls_value(int kind, const double* par, const double x[3]) {
    switch (kind) {
        case ORC_LS_SPHERE: { /* Sphere::dist (Surface.hpp:71), centred */
            double y[3] = {x[0] - par[0], x[1] - par[1], x[2] - par[2]};
            return norm3(y) - par[3];
        }
        case ORC_LS_TORUS: { /* Torus::dist (Surface.hpp:130) with r_min == r_max */
            int ax = (int)par[2];
            int a0 = (ax + 1) % 3, a1 = (ax + 2) % 3;
            double rho = sqrt(x[a0] * x[a0] + x[a1] * x[a1]) - par[0];
            return sqrt(rho * rho + x[ax] * x[ax]) - par[1];
        }
        case ORC_LS_ELLIPSOID: {
            double d[3] = {x[0] - par[0], x[1] - par[1], x[2] - par[2]};
            const double* R = par + 6;
            double y[3];
            for (int i = 0; i < 3; ++i) y[i] = (R[0 * 3 + i] * d[0] + R[1 * 3 + i] * d[1]) + R[2 * 3 + i] * d[2];
            double z[3] = {y[0] / par[3], y[1] / par[4], y[2] / par[5]};
            return norm3(z) - 1.0;
        }
        case ORC_LS_PLANE:
            return ((par[0] * x[0] + par[1] * x[1]) + par[2] * x[2]) - par[3];
    }
    return NAN;
}

void orc_levelset(int kind, const double* par, int p2, int64_t nv, int64_t ne, const double* coords,
                  const int32_t* edge_v, double* ls_vert, double* ls_edge) {
    for (int64_t v = 0; v < nv; ++v) ls_vert[v] = orc_ls_value(kind, par, coords + 3 * v);
    for (int64_t e = 0; e < ne; ++e) {
        int32_t a = edge_v[2 * e], b = edge_v[2 * e + 1];
        if (!p2) {
            ls_edge[e] = 0.5 * (ls_vert[a] + ls_vert[b]);
        } else {
            double m[3];
            for (int c = 0; c < 3; ++c) m[c] = 0.5 * (coords[3 * a + c] + coords[3 * b + c]);
            ls_edge[e] = orc_ls_value(kind, par, m);
        }
    }
}

/* ======================================================================= */
/* DOF numbering                                                             */
/* ======================================================================= */
static int sgn(double v) { return (v > 0.) - (v < 0.); }

/* distance() (geom/subtriangulation.tpp:38-46): returns 0 for a cut tet,
 * min |v| for a one-signed tet, -1 for an exact zero in a cut tet.        */
static double tet_distance(const double* f, int n) {
    int sum = 0;
    for (int i = 0; i < n; ++i) sum += sgn(f[i]);
    if (abs(sum) == n) {
        double m = fabs(f[0]);
        for (int i = 1; i < n; ++i)
            if (fabs(f[i]) < m) m = fabs(f[i]);
        return m;
    }
    for (int i = 0; i < n; ++i)
        if (f[i] == 0.) return -1.;
    return 0.;
}

static void gather_ls10(const int32_t* tv, const int32_t* te, const double* ls_vert, const double* ls_edge,
                        double out[10]) {
    for (int i = 0; i < 4; ++i) out[i] = ls_vert[tv[i]];
    for (int i = 0; i < 6; ++i) out[4 + i] = ls_edge[te[i]];
}

int orc_distribute_dofs(int64_t nt, const int32_t* tet_v, const int32_t* tet_e, int64_t nv, int64_t ne,
                        const double* ls_vert, const double* ls_edge, int p2, double dist, int64_t* n_active,
                        int64_t* n_dofs, int32_t* dof_vert, int32_t* dof_edge, uint8_t* active) {
    for (int64_t v = 0; v < nv; ++v) dof_vert[v] = -1;
    if (p2)
        for (int64_t e = 0; e < ne; ++e) dof_edge[e] = -1;
    /* the distance test of every tet on all threads (independent per tet);
       the first-touch numbering below stays serial in tet order, as the
       reference's */
    const int nth = g_threads > 0 ? g_threads : omp_get_max_threads();
    int zero = 0;
#pragma omp parallel for num_threads(nth) schedule(static) reduction(| : zero)
    for (int64_t t = 0; t < nt; ++t) {
        double f[10];
        gather_ls10(tet_v + 4 * t, tet_e + 6 * t, ls_vert, ls_edge, f);
        const double d = tet_distance(f, 10);
        zero |= d < 0.;
        active[t] = d >= 0. && d <= dist;
    }
    if (zero) return ORC_ERR_ZERO_NODE;
    int64_t na = 0, block = 0;
    for (int64_t t = 0; t < nt; ++t) {
        if (active[t]) {
            ++na;
            active[t] = 1;
            for (int i = 0; i < 4; ++i) {
                int32_t* slot = &dof_vert[tet_v[4 * t + i]];
                if (*slot < 0) *slot = (int32_t)block++;
            }
            if (p2)
                for (int i = 0; i < 6; ++i) {
                    int32_t* slot = &dof_edge[tet_e[6 * t + i]];
                    if (*slot < 0) *slot = (int32_t)block++;
                }
        }
    }
    *n_active = na;
    *n_dofs = block;
    return ORC_OK;
}

/* ======================================================================= */
/* principal lattice of order 2 and the surface patch                        */
/* ======================================================================= */
/* PrincipalLatticeCL (geom/principallattice.cpp:33-79) for n = 2.          */
static int lat_index(int i, int j, int k) {
    return (i > 0 ? ((i + 2) * (i + 1) * i) / 6 : 0) + (j > 0 ? ((j + 1) * j) / 2 : 0) + k;
}
static int in_ref(const int v[3], int n) { return n >= v[0] && v[0] >= v[1] && v[1] >= v[2]; }

void orc_lattice2(double verts[10][4], int tets[8][4]) {
    const int n = 2;
    int nv = 0;
    for (int x = 0; x <= n; ++x)
        for (int y = 0; y <= x; ++y)
            for (int z = 0; z <= y; ++z, ++nv) {
                verts[nv][0] = (double)(n - x) / n;
                verts[nv][1] = (double)(x - y) / n;
                verts[nv][2] = (double)(y - z) / n;
                verts[nv][3] = (double)z / n;
            }
    static const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    int nt = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j)
            for (int k = 0; k <= j; ++k)
                for (int l = 0; l < 6; ++l) {
                    int t[4][3] = {{i, j, k}};
                    int ok = 1;
                    for (int s = 1; s < 4 && ok; ++s) {
                        memcpy(t[s], t[s - 1], sizeof t[s]);
                        ++t[s][perm[l][s - 1]];
                        ok = in_ref(t[s], n);
                    }
                    if (!ok) continue;
                    for (int s = 0; s < 4; ++s) tets[nt][s] = lat_index(t[s][0], t[s][1], t[s][2]);
                    ++nt;
                }
}

/* P2 local dof -> lattice vertex (geom/principallattice.cpp p2_dof_on_lattice_2) */
static const int P2_ON_LAT[10] = {0, 4, 7, 9, 1, 2, 5, 3, 6, 8};

/* SPatchCL<3>::make_patch<MergeCutPolicyCL> on a principal lattice with nsub
 * sub-tets LT over the lattice vertices LV, level set lat_ls at the vertices */
static int make_patch_lat(int nsub, const double (*LV)[4], const int (*LT)[4], const double* lat_ls, orc_patch_t* p) {
    /* MergeCut memo: lattice edge (lo,hi) -> cut vertex number */
    int cut_key[ORC_MAX_PVERTS][2];
    double cut_bary[ORC_MAX_PVERTS][4];
    int n_cut = 0;
    int copied[10];
    for (int k = 0; k < 10; ++k) copied[k] = -1;
    double zero_bary[10][4];
    int n_zero = 0;
    int zuse_f[3 * ORC_MAX_FACETS], zuse_j[3 * ORC_MAX_FACETS], n_zuse = 0;

    p->n_facets = 0;
    for (int s = 0; s < nsub; ++s) {
        double loc[4];
        int sg[4], sum = 0;
        for (int k = 0; k < 4; ++k) {
            loc[k] = lat_ls[LT[s][k]];
            sg[k] = sgn(loc[k]);
            sum += sg[k];
        }
        /* SignTraitsCL<3>::assign / compute_cuts (geom/signtraits.h:112-139) */
        int cut[4], n_root = 0, n_root_vert = 0;
        if (sg[0] == 0 && sg[1] == 0 && sg[2] == 0 && sg[3] == 0) return ORC_ERR_ZERO_PATTERN;
        if (abs(sum) != 4) {
            for (int k = 0; k < 4; ++k)
                if (sg[k] == 0) cut[n_root_vert++] = k;
            n_root = n_root_vert;
            for (int e = 0; e < 6; ++e)
                if (sg[EV[e][0]] * sg[EV[e][1]] == -1) cut[n_root++] = e + 4;
        }
        /* RefPatchBuilderCL<3>::assign (geom/reftetracut.cpp:53-60) */
        if (n_root < 3) continue;
        int bnd = (n_root_vert == 3);
        for (int f = 0; f + 2 < n_root; ++f) {
            if (p->n_facets >= ORC_MAX_FACETS) return ORC_ERR_CAPACITY;
            int fi = p->n_facets++;
            p->boundary[fi] = bnd;
            /* make_sub_facet (geom/subtriangulation.tpp:146-177) */
            for (int j = 0; j < 3; ++j) {
                int lv = cut[f + j];
                if (lv < 4) {
                    int lat = LT[s][lv];
                    if (copied[lat] < 0) {
                        copied[lat] = n_zero;
                        memcpy(zero_bary[n_zero], LV[lat], sizeof zero_bary[0]);
                        ++n_zero;
                    }
                    p->facet[fi][j] = copied[lat];
                    zuse_f[n_zuse] = fi;
                    zuse_j[n_zuse] = j;
                    ++n_zuse;
                } else {
                    int v0 = EV[lv - 4][0], v1 = EV[lv - 4][1];
                    int a = LT[s][v0], b = LT[s][v1];
                    int lo = a < b ? a : b, hi = a < b ? b : a;
                    int id = -1;
                    for (int q = 0; q < n_cut; ++q)
                        if (cut_key[q][0] == lo && cut_key[q][1] == hi) { id = q; break; }
                    if (id < 0) {
                        if (n_cut >= ORC_MAX_PVERTS) return ORC_ERR_CAPACITY;
                        id = n_cut++;
                        cut_key[id][0] = lo;
                        cut_key[id][1] = hi;
                        /* MergeCutPolicyCL::operator() (geom/subtriangulation.h:514-524) */
                        double t = loc[v0] / (loc[v0] - loc[v1]);
                        for (int c = 0; c < 4; ++c) cut_bary[id][c] = (1.0 - t) * LV[a][c] + t * LV[b][c];
                    }
                    p->facet[fi][j] = id;
                }
            }
        }
    }
    for (int u = 0; u < n_zuse; ++u) p->facet[zuse_f[u]][zuse_j[u]] += n_cut;
    if (n_cut + n_zero > ORC_MAX_PVERTS) return ORC_ERR_CAPACITY;
    for (int q = 0; q < n_cut; ++q) memcpy(p->bary[q], cut_bary[q], sizeof p->bary[0]);
    for (int q = 0; q < n_zero; ++q) memcpy(p->bary[n_cut + q], zero_bary[q], sizeof p->bary[0]);
    p->n_cut_verts = n_cut;
    p->n_verts = n_cut + n_zero;
    return ORC_OK;
}

int orc_make_patch(const double ls10[10], orc_patch_t* p) {
    double LV[10][4];
    int LT[8][4];
    orc_lattice2(LV, LT);
    double lat_ls[10];
    for (int k = 0; k < 10; ++k) lat_ls[P2_ON_LAT[k]] = ls10[k];
    return make_patch_lat(8, (const double(*)[4])LV, (const int(*)[4])LT, lat_ls, p);
}

/* the patch on PrincipalLatticeCL::instance(1): the tet itself, its 4 vertices */
int orc_make_patch1(const double ls4[4], orc_patch_t* p) {
    static const double LV[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    static const int LT[1][4] = {{0, 1, 2, 3}};
    return make_patch_lat(1, LV, LT, ls4, p);
}

/* ======================================================================= */
/* quadrature rules (num/discretize.cpp:153-294)                             */
/* ======================================================================= */
static double Q2D_NODE[7][3], Q2D_W[7], Q3D_NODE[15][4], Q3D_W[15];
static int q_init = 0;
static void init_quad(void) {
    if (q_init) return;
    const double s15 = sqrt(15.0);
    /* Quad5_2DDataCL */
    Q2D_NODE[0][0] = Q2D_NODE[0][1] = Q2D_NODE[0][2] = 1. / 3.;
    double A1 = (6.0 - s15) / 21.0, B1 = (9.0 + 2.0 * s15) / 21.0;
    double A2 = (6.0 + s15) / 21.0, B2 = (9.0 - 2.0 * s15) / 21.0;
    double n2[6][3] = {{A1, A1, B1}, {A1, B1, A1}, {B1, A1, A1}, {A2, A2, B2}, {A2, B2, A2}, {B2, A2, A2}};
    for (int i = 0; i < 6; ++i) memcpy(Q2D_NODE[i + 1], n2[i], sizeof n2[i]);
    Q2D_W[0] = 9. / 80.;
    for (int i = 1; i <= 3; ++i) Q2D_W[i] = (155. - s15) / 2400.;
    for (int i = 4; i <= 6; ++i) Q2D_W[i] = (155. + s15) / 2400.;
    /* Quad5DataCL */
    for (int c = 0; c < 4; ++c) Q3D_NODE[0][c] = 0.25;
    double a1 = (7.0 - s15) / 34.0, b1 = (13.0 + 3.0 * s15) / 34.0;
    double a2 = (7.0 + s15) / 34.0, b2 = (13.0 - 3.0 * s15) / 34.0;
    double a3 = (10.0 - 2.0 * s15) / 40.0, b3 = (10.0 + 2.0 * s15) / 40.0;
    double n3[14][4] = {{a1, a1, a1, b1}, {a1, a1, b1, a1}, {a1, b1, a1, a1}, {b1, a1, a1, a1},
                        {a2, a2, a2, b2}, {a2, a2, b2, a2}, {a2, b2, a2, a2}, {b2, a2, a2, a2},
                        {a3, a3, b3, b3}, {a3, b3, a3, b3}, {a3, b3, b3, a3}, {b3, a3, a3, b3},
                        {b3, a3, b3, a3}, {b3, b3, a3, a3}};
    for (int i = 0; i < 14; ++i) memcpy(Q3D_NODE[i + 1], n3[i], sizeof n3[i]);
    Q3D_W[0] = 0.01975308641975308641975308641975308641975;
    for (int i = 1; i <= 4; ++i) Q3D_W[i] = 0.01198951396316977000173064248499538621936;
    for (int i = 5; i <= 8; ++i) Q3D_W[i] = 0.01151136787104539754677023934921978132914;
    for (int i = 9; i <= 14; ++i) Q3D_W[i] = 0.008818342151675485008818342151675485008818;
    q_init = 1;
}

/* ======================================================================= */
/* local forms: LocalAssembler (surfactant/ifacetransp.h:1013-1076,1242-1256, */
/* 1522-1589)                                                               */
/* ======================================================================= */
/* GetTrafoTr (geom/multigrid.h:603-623): T = J^{-T}, det = det J */
static void trafo(const double xv[4][3], double T[3][3], double* det) {
    double M[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) M[j][i] = xv[i + 1][j] - xv[0][j];
    double d = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
               M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
    T[0][0] = (M[1][1] * M[2][2] - M[1][2] * M[2][1]) / d;
    T[0][1] = (M[2][0] * M[1][2] - M[1][0] * M[2][2]) / d;
    T[0][2] = (M[1][0] * M[2][1] - M[2][0] * M[1][1]) / d;
    T[1][0] = (M[2][1] * M[0][2] - M[0][1] * M[2][2]) / d;
    T[1][1] = (M[0][0] * M[2][2] - M[2][0] * M[0][2]) / d;
    T[1][2] = (M[2][0] * M[0][1] - M[0][0] * M[2][1]) / d;
    T[2][0] = (M[0][1] * M[1][2] - M[1][1] * M[0][2]) / d;
    T[2][1] = (M[1][0] * M[0][2] - M[0][0] * M[1][2]) / d;
    T[2][2] = (M[0][0] * M[1][1] - M[1][0] * M[0][1]) / d;
    *det = d;
}

/* world gradients of the barycentric coordinates: grad lambda_i = T * gref_i */
static void bary_grads(const double T[3][3], double g[4][3]) {
    static const double gref[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 4; ++i)
        for (int r = 0; r < 3; ++r) g[i][r] = T[r][0] * gref[i][0] + T[r][1] * gref[i][1] + T[r][2] * gref[i][2];
}

/* P2 basis values (FE_P2CL::H0..H9, num/fe.h:288-297) */
static void p2_vals(const double b[4], double h[10]) {
    for (int i = 0; i < 4; ++i) h[i] = b[i] * (2. * b[i] - 1.);
    for (int e = 0; e < 6; ++e) h[4 + e] = 4. * b[EV[e][0]] * b[EV[e][1]];
}
/* world gradients of the P2 basis at barycentric point b */
static void p2_grads(const double b[4], const double gl[4][3], double g[10][3]) {
    for (int i = 0; i < 4; ++i)
        for (int r = 0; r < 3; ++r) g[i][r] = (4. * b[i] - 1.) * gl[i][r];
    for (int e = 0; e < 6; ++e) {
        int a = EV[e][0], c = EV[e][1];
        for (int r = 0; r < 3; ++r) g[4 + e][r] = 4. * (b[c] * gl[a][r] + b[a] * gl[c][r]);
    }
}
static void unit_normal(const double ls10[10], const double g[10][3], double n[3]) {
    double v[3] = {0, 0, 0};
    for (int k = 0; k < 10; ++k)
        for (int r = 0; r < 3; ++r) v[r] += ls10[k] * g[k][r];
    double nn = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int r = 0; r < 3; ++r) n[r] = v[r] / nn;
}
static double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

static double rhs_value(const orc_assemble_opts* o, const double x[3]) {
    if (o->rhs_kind == ORC_RHS_CONST) return o->rhs_par[0];
    if (o->rhs_kind == ORC_RHS_SPHERE_XYZ) {
        /* f(ext(x)), ext(x) = x - dist(x) * grad dist(x) (Surface.hpp:46-52) */
        double d[3] = {x[0] - o->rhs_par[0], x[1] - o->rhs_par[1], x[2] - o->rhs_par[2]};
        double nd = norm3(d);
        double dist = nd - o->rhs_par[3];
        double y[3];
        for (int c = 0; c < 3; ++c) y[c] = x[c] - dist * (d[c] / nd);
        return o->rhs_par[4] * y[0] * y[1] * y[2];
    }
    return 0.;
}

int orc_local_forms(const double xv[4][3], const double ls10[10], const orc_assemble_opts* o,
                    const double* chi_loc, const double* wind_loc, double out[ORC_NUM_MAT_FORMS][100],
                    double rhs[10], int* n_facets) {
    init_quad();
    const int nl = o->p2 ? 10 : 4;
    const int wantN = (o->forms & (1u << ORC_FORM_N)) != 0;
    if (wantN && (o->p2 || !wind_loc)) return ORC_ERR_BAD_INPUT;
    for (int f = 0; f < ORC_NUM_MAT_FORMS; ++f) memset(out[f], 0, sizeof(double) * 100);
    if (rhs) memset(rhs, 0, sizeof(double) * 10);
    orc_patch_t P;
    int st = orc_make_patch(ls10, &P);
    if (st) return st;
    if (n_facets) *n_facets = P.n_facets;
    double T[3][3], det;
    trafo(xv, T, &det);
    double absdet = fabs(det);
    double gl[4][3];
    bary_grads(T, gl);

    /* surface quadrature: make_CompositeQuadDomainCodim1 (num/quadrature.tpp:265-314) */
    for (int f = 0; f < P.n_facets; ++f) {
        double w[3][3];
        for (int j = 0; j < 3; ++j) {
            const double* b = P.bary[P.facet[f][j]];
            for (int c = 0; c < 3; ++c) w[j][c] = xv[0][c] * b[0] + xv[1][c] * b[1] + xv[2][c] * b[2] + xv[3][c] * b[3];
        }
        double u[3], v[3], cr[3];
        for (int c = 0; c < 3; ++c) { u[c] = w[1][c] - w[0][c]; v[c] = w[2][c] - w[0][c]; }
        cr[0] = u[1] * v[2] - u[2] * v[1];
        cr[1] = u[2] * v[0] - u[0] * v[2];
        cr[2] = u[0] * v[1] - u[1] * v[0];
        double fdet = norm3(cr) * (P.boundary[f] ? 0.5 : 1.0);
        for (int q = 0; q < 7; ++q) {
            double b[4];
            for (int c = 0; c < 4; ++c)
                b[c] = P.bary[P.facet[f][0]][c] * Q2D_NODE[q][0] + P.bary[P.facet[f][1]][c] * Q2D_NODE[q][1] +
                       P.bary[P.facet[f][2]][c] * Q2D_NODE[q][2];
            double wq = fdet * Q2D_W[q];
            double g2[10][3], n[3];
            p2_grads(b, gl, g2);
            unit_normal(ls10, g2, n);
            double phi[10], grad[10][3], sg[10][3];
            if (o->p2) {
                p2_vals(b, phi);
                memcpy(grad, g2, sizeof grad);
            } else {
                for (int i = 0; i < 4; ++i) { phi[i] = b[i]; memcpy(grad[i], gl[i], sizeof grad[i]); }
            }
            for (int i = 0; i < nl; ++i) {
                double gn = dot3(grad[i], n);
                for (int r = 0; r < 3; ++r) sg[i][r] = grad[i][r] - gn * n[r];
            }
            double mob = 1.0;
            if (chi_loc && o->degenerate) {
                double c = chi_loc[0] * b[0] + chi_loc[1] * b[1] + chi_loc[2] * b[2] + chi_loc[3] * b[3];
                mob = c * (1. - c);
                if (mob < 0.) mob = 0.;
            }
            for (int i = 0; i < nl; ++i)
                for (int j = i; j < nl; ++j) {
                    if (o->forms & (1u << ORC_FORM_M)) out[ORC_FORM_M][i * nl + j] += wq * (phi[j] * phi[i]);
                    double a = dot3(sg[j], sg[i]);
                    if (o->forms & (1u << ORC_FORM_A)) out[ORC_FORM_A][i * nl + j] += wq * a;
                    if (o->forms & (1u << ORC_FORM_LAPM)) out[ORC_FORM_LAPM][i * nl + j] += wq * (mob * a);
                }
            /* N_P1P1 (surfactant/ifacetransp.h:1590-1600): the P2 wind at the
               point (LocalP2CL evaluated there, buildWindCH :1129-1137) dotted
               with the surface gradient of phi_j, times phi_i */
            if (wantN) {
                double h[10], wnd[3] = {0., 0., 0.};
                p2_vals(b, h);
                for (int k = 0; k < 10; ++k)
                    for (int r = 0; r < 3; ++r) wnd[r] += wind_loc[3 * k + r] * h[k];
                for (int i = 0; i < 4; ++i)
                    for (int j = 0; j < 4; ++j) out[ORC_FORM_N][i * 4 + j] += wq * (dot3(wnd, sg[j]) * phi[i]);
            }
            if (rhs && o->rhs_kind != ORC_RHS_NONE) {
                double x[3];
                for (int c = 0; c < 3; ++c) x[c] = xv[0][c] * b[0] + xv[1][c] * b[1] + xv[2][c] * b[2] + xv[3][c] * b[3];
                double fx = rhs_value(o, x);
                for (int i = 0; i < nl; ++i) rhs[i] += wq * (fx * phi[i]);
            }
        }
    }
    /* volume stabilisation: C_n_P1P1 / diagonal block of C_n_vecP2vecP2 */
    if (o->forms & (1u << ORC_FORM_CN)) {
        double acc[100];
        memset(acc, 0, sizeof acc);
        for (int q = 0; q < 15; ++q) {
            const double* b = Q3D_NODE[q];
            double g2[10][3], n[3];
            p2_grads(b, gl, g2);
            unit_normal(ls10, g2, n);
            double dn[10];
            for (int i = 0; i < nl; ++i) dn[i] = o->p2 ? dot3(n, g2[i]) : dot3(n, gl[i]);
            for (int i = 0; i < nl; ++i)
                for (int j = i; j < nl; ++j) acc[i * nl + j] += Q3D_W[q] * (dn[j] * dn[i]);
        }
        for (int i = 0; i < nl; ++i)
            for (int j = i; j < nl; ++j) out[ORC_FORM_CN][i * nl + j] = acc[i * nl + j] * absdet;
    }
    for (int f = 0; f < ORC_NUM_MAT_FORMS; ++f) {
        if (f == ORC_FORM_N) continue; /* the only form that is not symmetric */
        for (int i = 0; i < nl; ++i)
            for (int j = 0; j < i; ++j) out[f][i * nl + j] = out[f][j * nl + i];
    }
    return ORC_OK;
}

/* ======================================================================= */
/* assembly into CSR: FESystemAccumulator + SparseMatBuilderCL::Build         */
/* ======================================================================= */
static int cmp_i32(const void* a, const void* b) {
    int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return (x > y) - (x < y);
}

static int64_t find_col(const int32_t* cols, int64_t lo, int64_t hi, int32_t c) {
    while (lo < hi) {
        int64_t mid = (lo + hi) / 2;
        if (cols[mid] < c) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

static void tet_dofs(const int32_t* tv, const int32_t* te, const int32_t* dof_vert, const int32_t* dof_edge,
                     int p2, int32_t I[10]) {
    for (int i = 0; i < 4; ++i) I[i] = dof_vert[tv[i]];
    if (p2)
        for (int i = 0; i < 6; ++i) I[4 + i] = dof_edge[te[i]];
}

int orc_assemble(int64_t nt, const int32_t* tet_v, const int32_t* tet_e, const double* coords,
                 const double* ls_vert, const double* ls_edge, const uint8_t* active, const int32_t* dof_vert,
                 const int32_t* dof_edge, int64_t m, const orc_assemble_opts* o, int64_t* rowptr,
                 int32_t** colind_out, int64_t* nnz_out, double* vals[ORC_NUM_MAT_FORMS], double* rhs) {
    const int nl = o->p2 ? 10 : 4;
    /* pattern: count with duplicates, then sort/unique per row */
    int64_t* cnt = (int64_t*)calloc((size_t)m + 1, sizeof(int64_t));
    for (int64_t t = 0; t < nt; ++t) {
        if (!active[t]) continue;
        int32_t I[10];
        tet_dofs(tet_v + 4 * t, tet_e + 6 * t, dof_vert, dof_edge, o->p2, I);
        for (int i = 0; i < nl; ++i) {
            if (I[i] < 0 || I[i] >= m) {
                free(cnt);
                return ORC_ERR_BAD_INPUT;
            }
            cnt[I[i] + 1] += nl;
        }
    }
    for (int64_t r = 0; r < m; ++r) cnt[r + 1] += cnt[r];
    int32_t* tmp = (int32_t*)malloc(sizeof(int32_t) * (size_t)(cnt[m] > 0 ? cnt[m] : 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m + 1));
    memcpy(fill, cnt, sizeof(int64_t) * (size_t)(m + 1));
    for (int64_t t = 0; t < nt; ++t) {
        if (!active[t]) continue;
        int32_t I[10];
        tet_dofs(tet_v + 4 * t, tet_e + 6 * t, dof_vert, dof_edge, o->p2, I);
        for (int i = 0; i < nl; ++i)
            for (int j = 0; j < nl; ++j) tmp[fill[I[i]]++] = I[j];
    }
    const int nth = g_threads > 0 ? g_threads : omp_get_max_threads();
    rowptr[0] = 0;
#pragma omp parallel for num_threads(nth) schedule(dynamic, 256)
    for (int64_t r = 0; r < m; ++r) {
        int64_t b = cnt[r], e = cnt[r + 1];
        qsort(tmp + b, (size_t)(e - b), sizeof(int32_t), cmp_i32);
        int64_t u = 0;
        for (int64_t k = b; k < e; ++k)
            if (k == b || tmp[k] != tmp[k - 1]) ++u;
        rowptr[r + 1] = u;
    }
    for (int64_t r = 0; r < m; ++r) rowptr[r + 1] += rowptr[r];
    int64_t nnz = rowptr[m];
    int32_t* colind = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
#pragma omp parallel for num_threads(nth) schedule(static)
    for (int64_t r = 0; r < m; ++r) {
        int64_t b = cnt[r], e = cnt[r + 1], w = rowptr[r];
        for (int64_t k = b; k < e; ++k)
            if (k == b || tmp[k] != tmp[k - 1]) colind[w++] = tmp[k];
    }
    free(tmp);
    free(fill);
    free(cnt);
    for (int f = 0; f < ORC_NUM_MAT_FORMS; ++f) {
        vals[f] = NULL;
        if (o->forms & (1u << f)) vals[f] = (double*)calloc((size_t)(nnz > 0 ? nnz : 1), sizeof(double));
    }
    if (rhs)
        for (int64_t r = 0; r < m; ++r) rhs[r] = 0.;
    /* values: the element matrices of all active tets on all threads (each
       depends on its tet only, like the reference's colour-class loop,
       num/accumulator.h:161-190), then accumulated serially in triangulation
       order, so the sums do not depend on the thread count */
    int64_t na = 0;
    for (int64_t t = 0; t < nt; ++t) na += active[t] != 0;
    int64_t* tl = (int64_t*)malloc(sizeof(int64_t) * (size_t)(na > 0 ? na : 1));
    na = 0;
    for (int64_t t = 0; t < nt; ++t)
        if (active[t]) tl[na++] = t;
    int fl[ORC_NUM_MAT_FORMS], nfl = 0;
    for (int f = 0; f < ORC_NUM_MAT_FORMS; ++f)
        if (vals[f]) fl[nfl++] = f;
    const int64_t stride = (int64_t)nfl * nl * nl + nl;
    double* E = (double*)malloc(sizeof(double) * (size_t)(na > 0 ? na * stride : 1));
    int64_t err_at = na;
    int err_st = 0;
    init_quad();
#pragma omp parallel for num_threads(nth) schedule(dynamic, 64)
    for (int64_t q = 0; q < na; ++q) {
        const int64_t t = tl[q];
        int32_t I[10];
        tet_dofs(tet_v + 4 * t, tet_e + 6 * t, dof_vert, dof_edge, o->p2, I);
        double xv[4][3], ls10[10];
        for (int i = 0; i < 4; ++i) memcpy(xv[i], coords + 3 * tet_v[4 * t + i], sizeof xv[i]);
        gather_ls10(tet_v + 4 * t, tet_e + 6 * t, ls_vert, ls_edge, ls10);
        double chi_loc[4], wind_loc[30], loc[ORC_NUM_MAT_FORMS][100], b[10];
        if (o->chi)
            for (int i = 0; i < 4; ++i) chi_loc[i] = o->chi[I[i]];
        const int haveW = o->wind_vert && o->wind_edge;
        if (haveW) {
            for (int k = 0; k < 4; ++k)
                for (int r = 0; r < 3; ++r) wind_loc[3 * k + r] = o->wind_vert[3 * (int64_t)tet_v[4 * t + k] + r];
            for (int k = 0; k < 6; ++k)
                for (int r = 0; r < 3; ++r)
                    wind_loc[3 * (4 + k) + r] = o->wind_edge[3 * (int64_t)tet_e[6 * t + k] + r];
        }
        int st = orc_local_forms(xv, ls10, o, o->chi ? chi_loc : NULL, haveW ? wind_loc : NULL, loc, b, NULL);
        if (st) {
#pragma omp critical(orc_assemble_err)
            if (q < err_at) {
                err_at = q;
                err_st = st;
            }
            continue;
        }
        double* e = E + q * stride;
        for (int k = 0; k < nfl; ++k) memcpy(e + (int64_t)k * nl * nl, loc[fl[k]], sizeof(double) * nl * nl);
        memcpy(e + (int64_t)nfl * nl * nl, b, sizeof(double) * nl);
    }
    if (err_at < na) {
        free(E);
        free(tl);
        free(colind);
        for (int f = 0; f < ORC_NUM_MAT_FORMS; ++f) { free(vals[f]); vals[f] = NULL; }
        return err_st;
    }
    for (int64_t q = 0; q < na; ++q) {
        const int64_t t = tl[q];
        int32_t I[10];
        tet_dofs(tet_v + 4 * t, tet_e + 6 * t, dof_vert, dof_edge, o->p2, I);
        const double* e = E + q * stride;
        for (int i = 0; i < nl; ++i) {
            int32_t r = I[i];
            for (int j = 0; j < nl; ++j) {
                int64_t pos = find_col(colind, rowptr[r], rowptr[r + 1], I[j]);
                for (int k = 0; k < nfl; ++k) vals[fl[k]][pos] += e[(int64_t)k * nl * nl + i * nl + j];
            }
            if (rhs && o->rhs_kind != ORC_RHS_NONE) rhs[r] += e[(int64_t)nfl * nl * nl + i];
        }
    }
    free(E);
    free(tl);
    *colind_out = colind;
    *nnz_out = nnz;
    return ORC_OK;
}

/* ======================================================================= */
/* legacy numbering CreateNumbOnInterfaceVertex (misc/problem.cpp:443-505)   */
/* ======================================================================= */
int orc_numb_on_interface_p1(int64_t nt, const int32_t* tet_v, const int32_t* tet_e, int64_t nv,
                             const double* coords, const double* ls_vert, const double* ls_edge, double omit_bound,
                             int64_t* n_active, int64_t* n_dofs, int32_t* dof_vert) {
    static const double Q2N[4][3] = {{1., 0., 0.}, {0., 1., 0.}, {0., 0., 1.}, {1. / 3., 1. / 3., 1. / 3.}};
    static const double Q2W[4] = {1. / 24., 1. / 24., 1. / 24., 0.375};
    for (int64_t v = 0; v < nv; ++v) dof_vert[v] = -1;
    int64_t counter = 0, na = 0;
    for (int64_t t = 0; t < nt; ++t) {
        double ls10[10], lat[10];
        gather_ls10(tet_v + 4 * t, tet_e + 6 * t, ls_vert, ls_edge, ls10);
        for (int k = 0; k < 10; ++k) lat[P2_ON_LAT[k]] = ls10[k];
        double d = tet_distance(lat, 10);
        if (d < 0.) return ORC_ERR_ZERO_NODE;
        if (d != 0.) continue;
        double xv[4][3];
        for (int i = 0; i < 4; ++i) memcpy(xv[i], coords + 3 * tet_v[4 * t + i], sizeof xv[i]);
        double T[3][3], det;
        trafo(xv, T, &det);
        double vol = fabs(det) / 6.;
        double limit = omit_bound < 0. ? 0. : omit_bound * pow(vol * 6, 4. / 3.);
        orc_patch_t P;
        int st = orc_make_patch(ls10, &P);
        if (st) return st;
        if (P.n_facets == 0) continue;
        int act = 0;
        for (int i = 0; i < 4; ++i) {
            int32_t* slot = &dof_vert[tet_v[4 * t + i]];
            if (*slot >= 0) { act = 1; continue; }
            /* coefficients of lambda_i^2 as a P2 function: 1 at vertex i, 1/4 on its edges */
            double c[10] = {0};
            c[i] = 1.;
            for (int e = 0; e < 6; ++e)
                if (EV[e][0] == i || EV[e][1] == i) c[4 + e] = 0.25;
            double s = 0.;
            for (int f = 0; f < P.n_facets; ++f) {
                double w[3][3];
                for (int j = 0; j < 3; ++j) {
                    const double* b = P.bary[P.facet[f][j]];
                    for (int cc = 0; cc < 3; ++cc)
                        w[j][cc] = xv[0][cc] * b[0] + xv[1][cc] * b[1] + xv[2][cc] * b[2] + xv[3][cc] * b[3];
                }
                double u[3], v[3], cr[3];
                for (int cc = 0; cc < 3; ++cc) { u[cc] = w[1][cc] - w[0][cc]; v[cc] = w[2][cc] - w[0][cc]; }
                cr[0] = u[1] * v[2] - u[2] * v[1];
                cr[1] = u[2] * v[0] - u[0] * v[2];
                cr[2] = u[0] * v[1] - u[1] * v[0];
                double fdet = norm3(cr) * (P.boundary[f] ? 0.5 : 1.0);
                for (int q = 0; q < 4; ++q) {
                    double b[4], h[10];
                    for (int cc = 0; cc < 4; ++cc)
                        b[cc] = P.bary[P.facet[f][0]][cc] * Q2N[q][0] + P.bary[P.facet[f][1]][cc] * Q2N[q][1] +
                                P.bary[P.facet[f][2]][cc] * Q2N[q][2];
                    p2_vals(b, h);
                    double val = 0.;
                    for (int k = 0; k < 10; ++k) val += c[k] * h[k];
                    s += (fdet * Q2W[q]) * val;
                }
            }
            if (s > limit) {
                *slot = (int32_t)counter++;
                act = 1;
            }
        }
        na += act;
    }
    *n_active = na;
    *n_dofs = counter;
    return ORC_OK;
}

/* ======================================================================= */
/* legacy P1 interface forms (surfactant.cpp path)                           */
/* ======================================================================= */
/* Children of the regular refinement in P2-DoF numbering (ChildDataAr,
 * geom/topo.cpp:333-341): vertices 0..3, edge midpoints 4 + edge.           */
static const int REG_CHILD[8][4] = {{0, 4, 5, 7}, {4, 1, 6, 8}, {4, 5, 6, 8}, {4, 5, 7, 8},
                                    {5, 6, 2, 9}, {5, 6, 8, 9}, {5, 7, 8, 9}, {7, 8, 9, 3}};

/* InterfacePatchCL::Sign (num/interfacePatch.h:75): |phi| < 2 eps counts as 0 */
static int legacy_sign(double phi) {
    const double approx_zero = 2. * 2.220446049250313e-16;
    return fabs(phi) < approx_zero ? 0 : (phi > 0 ? 1 : -1);
}

double orc_rhs_quadratic(const double* p, const double x[3]) {
    return ((p[0] + p[1] * x[0] + p[2] * x[1] + p[3] * x[2]) + (p[4] * x[0] * x[0] + p[5] * x[1] * x[1] + p[6] * x[2] * x[2])) +
           (p[7] * x[0] * x[1] + p[8] * x[0] * x[2] + p[9] * x[1] * x[2]);
}

/* Planar pieces of one regular child (InterfacePatchCL::ComputeVerticesOfCut,
 * num/interfacePatch.cpp:137-199, InterfaceTriangleCL::ComputeForChild,
 * :478-512): up to two triangles, barycentric in the parent, with |det|.
 * Returns the triangle count, -1 for a 3-dimensional zero level.           */
int orc_legacy_child_triangles(const double xv[4][3], const double ls10[10], int ch, double tri[2][3][4],
                               double det[2]) {
    double bdof[10][4], cdof[10][3];
    int sgn10[10];
    for (int v = 0; v < 10; ++v) {
        for (int c = 0; c < 4; ++c) bdof[v][c] = 0.;
        if (v < 4) {
            bdof[v][v] = 1.;
            for (int c = 0; c < 3; ++c) cdof[v][c] = xv[v][c];
        } else {
            const int a = EV[v - 4][0], b = EV[v - 4][1];
            bdof[v][a] = 0.5;
            bdof[v][b] = 0.5;
            for (int c = 0; c < 3; ++c) cdof[v][c] = 0.5 * (xv[a][c] + xv[b][c]);
        }
        sgn10[v] = legacy_sign(ls10[v]);
    }
    const int* cv = REG_CHILD[ch];
    int ns[3] = {0, 0, 0};
    for (int k = 0; k < 4; ++k) ++ns[sgn10[cv[k]] + 1];
    if (ns[0] * ns[2] == 0 && ns[1] < 3) return 0;
    if (ns[1] == 4) return -1;
    double bary[4][4], pqrs[4][3];
    int np = 0;
    for (int k = 0; k < 4; ++k) {
        const int v = cv[k];
        if (sgn10[v] == 0) {
            memcpy(bary[np], bdof[v], sizeof bary[np]);
            memcpy(pqrs[np], cdof[v], sizeof pqrs[np]);
            ++np;
        }
    }
    for (int e = 0; e < 6; ++e) {
        const int v0 = cv[EV[e][0]], v1 = cv[EV[e][1]];
        if (sgn10[v0] * sgn10[v1] < 0) {
            const double lam = ls10[v0] / (ls10[v0] - ls10[v1]);
            for (int c = 0; c < 4; ++c) bary[np][c] = (1. - lam) * bdof[v0][c] + lam * bdof[v1][c];
            for (int c = 0; c < 3; ++c) pqrs[np][c] = (1. - lam) * cdof[v0][c] + lam * cdof[v1][c];
            ++np;
        }
    }
    for (int f = 0; f < 4; ++f) {  /* cut lying on a face of the parent */
        int on = 0;
        for (int i = 0; i < np; ++i) on += bary[i][f] < 1e-9;
        if (on == np) return 0;
    }
    if (np < 3) return 0;
    double u[3], v[3], cr[3];
    for (int c = 0; c < 3; ++c) {
        u[c] = pqrs[1][c] - pqrs[0][c];
        v[c] = pqrs[2][c] - pqrs[0][c];
    }
    cr[0] = u[1] * v[2] - u[2] * v[1];
    cr[1] = u[2] * v[0] - u[0] * v[2];
    cr[2] = u[0] * v[1] - u[1] * v[0];
    double d = norm3(cr);
    if (ns[1] >= 3) d /= 2.; /* EqualToFace: the patch is shared by two children */
    for (int j = 0; j < 3; ++j) memcpy(tri[0][j], bary[j], sizeof tri[0][j]);
    det[0] = d;
    if (np < 4) return 1;
    /* |(Q-P) a + (R-P) b - (S-P)| -> min (normal equations) */
    double w[3];
    for (int c = 0; c < 3; ++c) w[c] = pqrs[3][c] - pqrs[0][c];
    const double uu = dot3(u, u), uv = dot3(u, v), vv = dot3(v, v), uw = dot3(u, w), vw = dot3(v, w);
    const double dd = uu * vv - uv * uv;
    const double aa = (uw * vv - vw * uv) / dd, bb = (vw * uu - uw * uv) / dd;
    for (int j = 0; j < 3; ++j) memcpy(tri[1][j], bary[j + 1], sizeof tri[1][j]);
    det[1] = d * (aa + bb - 1.);
    return 2;
}

int orc_legacy_local(const double xv[4][3], const double ls10[10], double alpha, double D, const double* fpar,
                     double mass[16], double lb[16], double rhs[4], int* nonempty) {
    init_quad();
    static const double Q2N[4][3] = {{1., 0., 0.}, {0., 1., 0.}, {0., 0., 1.}, {1. / 3., 1. / 3., 1. / 3.}};
    static const double Q2W[4] = {1. / 24., 1. / 24., 1. / 24., 0.375};
    for (int k = 0; k < 16; ++k) mass[k] = lb[k] = 0.;
    for (int k = 0; k < 4; ++k) rhs[k] = 0.;
    *nonempty = 0;
    /* matrices on the lattice-2 patch (InterfaceCommonDataP1CL::visit, ifacetransp.h:142-149) */
    orc_patch_t P;
    int st = orc_make_patch(ls10, &P);
    if (st) return st;
    double T[3][3], dett, gl[4][3];
    trafo(xv, T, &dett);
    bary_grads(T, gl);
    if (P.n_facets > 0) {
        *nonempty = 1;
        double qs[4][4] = {{0}};
        for (int f = 0; f < P.n_facets; ++f) {
            double wv[3][3];
            for (int j = 0; j < 3; ++j) {
                const double* b = P.bary[P.facet[f][j]];
                for (int c = 0; c < 3; ++c) wv[j][c] = xv[0][c] * b[0] + xv[1][c] * b[1] + xv[2][c] * b[2] + xv[3][c] * b[3];
            }
            double u[3], v[3], cr[3];
            for (int c = 0; c < 3; ++c) {
                u[c] = wv[1][c] - wv[0][c];
                v[c] = wv[2][c] - wv[0][c];
            }
            cr[0] = u[1] * v[2] - u[2] * v[1];
            cr[1] = u[2] * v[0] - u[0] * v[2];
            cr[2] = u[0] * v[1] - u[1] * v[0];
            const double ad = norm3(cr);
            /* mass: Quad2_2D composite rule, weights halved on lattice faces */
            const double wq = ad * (P.boundary[f] ? 0.5 : 1.);
            for (int q = 0; q < 4; ++q) {
                double b[4];
                for (int c = 0; c < 4; ++c)
                    b[c] = P.bary[P.facet[f][0]][c] * Q2N[q][0] + P.bary[P.facet[f][1]][c] * Q2N[q][1] +
                           P.bary[P.facet[f][2]][c] * Q2N[q][2];
                for (int i = 0; i < 4; ++i)
                    for (int j = 0; j < 4; ++j) qs[i][j] += (wq * Q2W[q]) * (b[i] * b[j]);
            }
            /* Laplace-Beltrami: facet normal, D/2 |det| (no halving) */
            if (ad > 0.) {
                double n[3] = {cr[0] / ad, cr[1] / ad, cr[2] / ad}, pq[4][3];
                for (int i = 0; i < 4; ++i) {
                    const double gn = dot3(gl[i], n);
                    for (int c = 0; c < 3; ++c) pq[i][c] = gl[i][c] - gn * n[c];
                }
                for (int i = 0; i < 4; ++i)
                    for (int j = 0; j < 4; ++j) lb[4 * i + j] += dot3(pq[i], pq[j]) * ad;
            }
        }
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) {
                mass[4 * i + j] = i == j ? qs[i][i] : alpha * qs[i][j];
                lb[4 * i + j] *= D * 0.5;
            }
    }
    /* rhs on the regular children (SetupInterfaceRhsP1, ifacetransp.cpp:532-563) */
    int sg0 = legacy_sign(ls10[0]), inter = 0;
    for (int v = 1; v < 10; ++v)
        if (legacy_sign(ls10[v]) != sg0) inter = 1;
    if (inter) {
        for (int ch = 0; ch < 8; ++ch) {
            double tri[2][3][4], det[2];
            const int nt = orc_legacy_child_triangles(xv, ls10, ch, tri, det);
            if (nt < 0) return ORC_ERR_ZERO_PATTERN;
            for (int t = 0; t < nt; ++t)
                for (int q = 0; q < 7; ++q) {
                    double b[4], x[3];
                    for (int c = 0; c < 4; ++c)
                        b[c] = tri[t][0][c] * Q2D_NODE[q][0] + tri[t][1][c] * Q2D_NODE[q][1] + tri[t][2][c] * Q2D_NODE[q][2];
                    for (int c = 0; c < 3; ++c) x[c] = xv[0][c] * b[0] + xv[1][c] * b[1] + xv[2][c] * b[2] + xv[3][c] * b[3];
                    const double fx = orc_rhs_quadratic(fpar, x);
                    for (int i = 0; i < 4; ++i) rhs[i] += (det[t] * Q2D_W[q]) * (fx * b[i]);
                }
        }
    }
    return ORC_OK;
}

int orc_assemble_legacy_p1(int64_t nt, const int32_t* tet_v, const int32_t* tet_e, const double* coords,
                           const double* ls_vert, const double* ls_edge, const int32_t* dof_vert, int64_t m,
                           double alpha, double D, const double* fpar, int64_t* rowptr, int32_t** colind_out,
                           int64_t* nnz_out, double** mass_out, double** lb_out, double* rhs) {
    uint8_t* vis = (uint8_t*)calloc((size_t)(nt > 0 ? nt : 1), 1);
    double(*loc)[36] = (double(*)[36])malloc(sizeof(double) * 36 * (size_t)(nt > 0 ? nt : 1));
    for (int64_t t = 0; t < nt; ++t) {
        double xv[4][3], ls10[10];
        for (int i = 0; i < 4; ++i) memcpy(xv[i], coords + 3 * tet_v[4 * t + i], sizeof xv[i]);
        gather_ls10(tet_v + 4 * t, tet_e + 6 * t, ls_vert, ls_edge, ls10);
        int ne = 0;
        int st = orc_legacy_local(xv, ls10, alpha, D, fpar, loc[t], loc[t] + 16, loc[t] + 32, &ne);
        if (st) {
            free(vis);
            free(loc);
            return st;
        }
        vis[t] = (uint8_t)ne;
    }
    /* pattern: numbered pairs of the visited tets (MatrixBuilderCL keeps explicit zeros) */
    int64_t* cnt = (int64_t*)calloc((size_t)m + 1, sizeof(int64_t));
    for (int64_t t = 0; t < nt; ++t) {
        if (!vis[t]) continue;
        for (int i = 0; i < 4; ++i) {
            const int32_t r = dof_vert[tet_v[4 * t + i]];
            if (r >= 0) cnt[r + 1] += 4;
        }
    }
    for (int64_t r = 0; r < m; ++r) cnt[r + 1] += cnt[r];
    int32_t* tmp = (int32_t*)malloc(sizeof(int32_t) * (size_t)(cnt[m] > 0 ? cnt[m] : 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m + 1));
    memcpy(fill, cnt, sizeof(int64_t) * (size_t)(m + 1));
    int64_t* ecnt = (int64_t*)calloc((size_t)m + 1, sizeof(int64_t));
    for (int64_t t = 0; t < nt; ++t) {
        if (!vis[t]) continue;
        for (int i = 0; i < 4; ++i) {
            const int32_t r = dof_vert[tet_v[4 * t + i]];
            if (r < 0) continue;
            for (int j = 0; j < 4; ++j) {
                const int32_t c = dof_vert[tet_v[4 * t + j]];
                if (c >= 0) tmp[fill[r]++] = c;
            }
        }
    }
    rowptr[0] = 0;
    for (int64_t r = 0; r < m; ++r) {
        const int64_t b = cnt[r], e = fill[r];
        qsort(tmp + b, (size_t)(e - b), sizeof(int32_t), cmp_i32);
        int64_t u = 0;
        for (int64_t k = b; k < e; ++k)
            if (k == b || tmp[k] != tmp[k - 1]) ++u;
        rowptr[r + 1] = rowptr[r] + u;
    }
    const int64_t nnz = rowptr[m];
    int32_t* colind = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nnz > 0 ? nnz : 1));
    for (int64_t r = 0; r < m; ++r) {
        int64_t w = rowptr[r];
        for (int64_t k = cnt[r]; k < fill[r]; ++k)
            if (k == cnt[r] || tmp[k] != tmp[k - 1]) colind[w++] = tmp[k];
    }
    free(tmp);
    free(fill);
    free(cnt);
    free(ecnt);
    double* M = (double*)calloc((size_t)(nnz > 0 ? nnz : 1), sizeof(double));
    double* A = (double*)calloc((size_t)(nnz > 0 ? nnz : 1), sizeof(double));
    for (int64_t r = 0; r < m; ++r) rhs[r] = 0.;
    for (int64_t t = 0; t < nt; ++t) {
        int32_t I[4];
        for (int i = 0; i < 4; ++i) I[i] = dof_vert[tet_v[4 * t + i]];
        for (int i = 0; i < 4; ++i)
            if (I[i] >= 0) rhs[I[i]] += loc[t][32 + i];
        if (!vis[t]) continue;
        for (int i = 0; i < 4; ++i) {
            if (I[i] < 0) continue;
            for (int j = 0; j < 4; ++j) {
                if (I[j] < 0) continue;
                const int64_t pos = find_col(colind, rowptr[I[i]], rowptr[I[i] + 1], I[j]);
                M[pos] += loc[t][4 * i + j];
                A[pos] += loc[t][16 + 4 * i + j];
            }
        }
    }
    free(vis);
    free(loc);
    *colind_out = colind;
    *nnz_out = nnz;
    *mass_out = M;
    *lb_out = A;
    return ORC_OK;
}

/* ======================================================================= */
/* sparse linear algebra and Krylov solvers                                  */
/* ======================================================================= */
void orc_spmv(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* vals, const double* x,
              double* y) {
#ifdef _OPENMP
    int nth = g_threads > 0 ? g_threads : omp_get_max_threads();
#pragma omp parallel for num_threads(nth) schedule(static)
#endif
    for (int64_t r = 0; r < m; ++r) {
        double s = 0.;
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) s += vals[k] * x[colind[k]];
        y[r] = s;
    }
}

/* KahanInnerProd (num/spmat.h:318-330) */
double orc_kahan_dot(int64_t n, const double* x, const double* y) {
    double sum = 0., c = 0., t, yy;
    for (int64_t i = 0; i < n; ++i) {
        yy = x[i] * y[i] - c;
        t = sum + yy;
        c = (t - sum) - yy;
        sum = t;
    }
    return sum;
}
static double plain_dot(int64_t n, const double* x, const double* y) {
    double s = 0.;
    for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
    return s;
}

/* diagonal found by a row scan (SolveGSstep<PB_JAC0>, num/precond.h:153-169) */
static void jacobi_diag(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* vals, double* d) {
    for (int64_t r = 0; r < m; ++r) {
        int64_t k = rowptr[r];
        while (k < rowptr[r + 1] && colind[k] != r) ++k;
        d[r] = k < rowptr[r + 1] ? vals[k] : 0.;
    }
}

int orc_pcg_jacobi(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* vals, const double* b,
                   double* x, int* max_iter, double* tol, int rel) {
    double* d = (double*)malloc(sizeof(double) * (size_t)m * 6);
    double *p = d + m, *z = p + m, *q = z + m, *r = q + m, *tmp = r + m;
    jacobi_diag(m, rowptr, colind, vals, d);
    orc_spmv(m, rowptr, colind, vals, x, tmp);
    for (int64_t i = 0; i < m; ++i) r[i] = b[i] - tmp[i];
    double resid = sqrt(orc_kahan_dot(m, r, r));
    double normb = sqrt(orc_kahan_dot(m, b, b));
    if (normb == 0.0 || !rel) normb = 1.0;
    resid = resid / normb;
    if (resid <= *tol) {
        *tol = resid;
        *max_iter = 0;
        free(d);
        return ORC_OK;
    }
    for (int64_t i = 0; i < m; ++i) z[i] = 1.0 * r[i] / d[i];
    double rho = orc_kahan_dot(m, z, r), rho_1;
    memcpy(p, z, sizeof(double) * (size_t)m);
    for (int it = 1; it <= *max_iter; ++it) {
        orc_spmv(m, rowptr, colind, vals, p, q);
        double lambda = orc_kahan_dot(m, q, p);
        double alpha = rho / lambda;
        for (int64_t i = 0; i < m; ++i) x[i] += alpha * p[i];
        for (int64_t i = 0; i < m; ++i) r[i] += (-alpha) * q[i];
        resid = sqrt(orc_kahan_dot(m, r, r)) / normb;
        if (resid <= *tol) {
            *tol = resid;
            *max_iter = it;
            free(d);
            return ORC_OK;
        }
        for (int64_t i = 0; i < m; ++i) z[i] = 1.0 * r[i] / d[i];
        rho_1 = rho;
        rho = orc_kahan_dot(m, z, r);
        double beta = rho / rho_1;
        for (int64_t i = 0; i < m; ++i) p[i] = z[i] + beta * p[i];
    }
    *tol = resid;
    free(d);
    return ORC_ERR_NOT_CONVERGED;
}

/* Nodal 2x2 block Jacobi for a 2x2 block system of size 2*h: the inverse of
 * [[a(i,i), a(i,i+h)], [a(i+h,i), a(i+h,i+h)]] applied to (v_i, v_{i+h}).   */
static void block_inv(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* vals, double* inv) {
    const int64_t h = m / 2;
    for (int64_t i = 0; i < h; ++i) {
        double a11 = 0, a12 = 0, a21 = 0, a22 = 0;
        for (int64_t k = rowptr[i]; k < rowptr[i + 1]; ++k) {
            if (colind[k] == i) a11 = vals[k];
            if (colind[k] == i + h) a12 = vals[k];
        }
        for (int64_t k = rowptr[i + h]; k < rowptr[i + h + 1]; ++k) {
            if (colind[k] == i) a21 = vals[k];
            if (colind[k] == i + h) a22 = vals[k];
        }
        const double det = a11 * a22 - a12 * a21;
        inv[4 * i] = a22 / det;
        inv[4 * i + 1] = -a12 / det;
        inv[4 * i + 2] = -a21 / det;
        inv[4 * i + 3] = a11 / det;
    }
}
static void prec_apply(int64_t m, int block, const double* d, const double* inv, const double* v, double* out) {
    if (!block) {
        for (int64_t i = 0; i < m; ++i) out[i] = v[i] / d[i];
        return;
    }
    const int64_t h = m / 2;
    for (int64_t i = 0; i < h; ++i) {
        const double a = v[i], c = v[i + h];
        out[i] = inv[4 * i] * a + inv[4 * i + 1] * c;
        out[i + h] = inv[4 * i + 2] * a + inv[4 * i + 3] * c;
    }
}

int orc_gmres_jacobi(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* vals, const double* b,
                     double* x, int restart, int* max_iter, double* tol, int rel, int method) {
    return orc_gmres(m, rowptr, colind, vals, b, x, restart, max_iter, tol, rel, method, 0);
}

int orc_gmres(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* vals, const double* b,
              double* x, int restart, int* max_iter, double* tol, int rel, int method, int block) {
    int mm = restart <= *max_iter ? restart : *max_iter;
    double* d = (double*)malloc(sizeof(double) * (size_t)m * (size_t)(mm + 7));
    double *w = d + m, *r = w + m, *t = r + m, *u = t + m, *inv = u + m, *V = inv + 2 * m;
    double* H = (double*)calloc((size_t)mm * mm, sizeof(double));
    double* s = (double*)calloc((size_t)mm, sizeof(double));
    double* cs = (double*)calloc((size_t)mm, sizeof(double));
    double* sn = (double*)calloc((size_t)mm, sizeof(double));
    double* y = (double*)calloc((size_t)mm, sizeof(double));
#define HH(i, j) H[(size_t)(i) * mm + (j)]
    jacobi_diag(m, rowptr, colind, vals, d);
    if (block) block_inv(m, rowptr, colind, vals, inv);
    double beta, normb, resid;
    orc_spmv(m, rowptr, colind, vals, x, t);
    if (method == 0) {
        for (int64_t i = 0; i < m; ++i) r[i] = b[i] - t[i];
        beta = sqrt(plain_dot(m, r, r));
        normb = sqrt(plain_dot(m, b, b));
    } else {
        for (int64_t i = 0; i < m; ++i) u[i] = b[i] - t[i];
        prec_apply(m, block, d, inv, u, r);
        beta = sqrt(plain_dot(m, r, r));
        prec_apply(m, block, d, inv, b, w);
        normb = sqrt(plain_dot(m, w, w));
    }
    if (normb == 0.0 || !rel) normb = 1.0;
    resid = beta / normb;
    int ret = ORC_ERR_NOT_CONVERGED;
    if (resid <= *tol) {
        *tol = resid;
        *max_iter = 0;
        ret = ORC_OK;
        goto done;
    }
    int j = 1;
    while (j <= *max_iter) {
        for (int64_t k = 0; k < m; ++k) V[k] = r[k] * (1.0 / beta);
        for (int k = 0; k < mm; ++k) s[k] = 0.;
        s[0] = beta;
        int i;
        for (i = 0; i < mm - 1 && j <= *max_iter; ++i, ++j) {
            double* vi = V + (size_t)i * m;
            if (method == 0) {
                prec_apply(m, block, d, inv, vi, t);
                orc_spmv(m, rowptr, colind, vals, t, w);
            } else {
                orc_spmv(m, rowptr, colind, vals, vi, t);
                prec_apply(m, block, d, inv, t, w);
            }
            for (int k = 0; k <= i; ++k) {
                double* vk = V + (size_t)k * m;
                HH(k, i) = plain_dot(m, w, vk);
                for (int64_t q = 0; q < m; ++q) w[q] -= HH(k, i) * vk[q];
            }
            HH(i + 1, i) = sqrt(plain_dot(m, w, w));
            double* vn = V + (size_t)(i + 1) * m;
            for (int64_t q = 0; q < m; ++q) vn[q] = w[q] * (1.0 / HH(i + 1, i));
            for (int k = 0; k < i; ++k) {
                double tmp = cs[k] * HH(k, i) + sn[k] * HH(k + 1, i);
                HH(k + 1, i) = -sn[k] * HH(k, i) + cs[k] * HH(k + 1, i);
                HH(k, i) = tmp;
            }
            /* GMRES_GeneratePlaneRotation / ApplyPlaneRotation (num/krylovsolver.h:263-282) */
            {
                double dx = HH(i, i), dy = HH(i + 1, i);
                if (dy == 0.0) { cs[i] = 1.0; sn[i] = 0.0; }
                else { double rr = sqrt(dx * dx + dy * dy); cs[i] = dx / rr; sn[i] = dy / rr; }
                double tmp = cs[i] * HH(i, i) + sn[i] * HH(i + 1, i);
                HH(i + 1, i) = -sn[i] * HH(i, i) + cs[i] * HH(i + 1, i);
                HH(i, i) = tmp;
                tmp = cs[i] * s[i] + sn[i] * s[i + 1];
                s[i + 1] = -sn[i] * s[i] + cs[i] * s[i + 1];
                s[i] = tmp;
            }
            resid = fabs(s[i + 1]) / normb;
            if (resid <= *tol) {
                int kk = i;
                for (int q = 0; q <= kk; ++q) y[q] = s[q];
                for (int q = kk; q >= 0; --q) {
                    y[q] /= HH(q, q);
                    for (int p = q - 1; p >= 0; --p) y[p] -= HH(p, q) * y[q];
                }
                if (method == 0) {
                    for (int64_t k = 0; k < m; ++k) w[k] = 0.;
                    for (int q = 0; q <= kk; ++q)
                        for (int64_t k = 0; k < m; ++k) w[k] += y[q] * V[(size_t)q * m + k];
                    prec_apply(m, block, d, inv, w, u);
                    for (int64_t k = 0; k < m; ++k) x[k] += u[k];
                } else {
                    for (int q = 0; q <= kk; ++q)
                        for (int64_t k = 0; k < m; ++k) x[k] += y[q] * V[(size_t)q * m + k];
                }
                *tol = resid;
                *max_iter = j;
                ret = ORC_OK;
                goto done;
            }
        }
        {
            int kk = i - 1;
            for (int q = 0; q <= kk; ++q) y[q] = s[q];
            for (int q = kk; q >= 0; --q) {
                y[q] /= HH(q, q);
                for (int p = q - 1; p >= 0; --p) y[p] -= HH(p, q) * y[q];
            }
            if (method == 0) {
                for (int64_t k = 0; k < m; ++k) w[k] = 0.;
                for (int q = 0; q <= kk; ++q)
                    for (int64_t k = 0; k < m; ++k) w[k] += y[q] * V[(size_t)q * m + k];
                prec_apply(m, block, d, inv, w, u);
                for (int64_t k = 0; k < m; ++k) x[k] += u[k];
                orc_spmv(m, rowptr, colind, vals, x, t);
                for (int64_t k = 0; k < m; ++k) r[k] = b[k] - t[k];
            } else {
                for (int q = 0; q <= kk; ++q)
                    for (int64_t k = 0; k < m; ++k) x[k] += y[q] * V[(size_t)q * m + k];
                orc_spmv(m, rowptr, colind, vals, x, t);
                for (int64_t k = 0; k < m; ++k) u[k] = b[k] - t[k];
                prec_apply(m, block, d, inv, u, r);
            }
        }
        beta = sqrt(plain_dot(m, r, r));
        resid = beta / normb;
        if (resid <= *tol) {
            *tol = resid;
            *max_iter = j;
            ret = ORC_OK;
            goto done;
        }
    }
    *tol = resid;
done:
#undef HH
    free(d);
    free(H);
    free(s);
    free(cs);
    free(sn);
    free(y);
    return ret;
}

int orc_ch_block(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* M, const double* A,
                 const double* C, const double* Amob, const double* N, double alpha, double mob, double rho,
                 double eps2, double beta, int64_t* browptr, int32_t* bcolind, double* bvals) {
    /* surfphasesep/surfphasesep.cpp:431-434: row r of the top blocks
       [alpha*M (+ N) | mob*Amob + rho*C] (Amob: A_deg or, when NULL, A_one);
       bottom: [eps2*A + beta*M + eps2*rho*C | -M] with A = A_one */
    if (!Amob) Amob = A;
    int64_t w = 0;
    browptr[0] = 0;
    for (int half = 0; half < 2; ++half)
        for (int64_t r = 0; r < m; ++r) {
            for (int blk = 0; blk < 2; ++blk)
                for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
                    double v;
                    if (half == 0) v = blk == 0 ? (N ? alpha * M[k] + N[k] : alpha * M[k]) : mob * Amob[k] + rho * C[k];
                    else v = blk == 0 ? (eps2 * A[k] + beta * M[k]) + (eps2 * rho) * C[k] : -1. * M[k];
                    bcolind[w] = (int32_t)(colind[k] + blk * m);
                    bvals[w] = v;
                    ++w;
                }
            browptr[half * m + r + 1] = w;
        }
    return ORC_OK;
}

/* ======================================================================= */
/* isoparametric P2 TraceFEM: the QuaQua mapper (levelset/levelsetmapper.cpp)  */
/* and LocalMassP2CL / LocalLaplaceBeltramiP2CL / LocalVectorP2CL              */
/* (surfactant/ifacetransp.h:2286-2402) on the linear interface              */
/* ======================================================================= */
/* averaging_P2_gradient_recovery (num/gradient_recovery.cpp:82-89,
 * OswaldProjectionP2AccuCL num/oswald_projection.h:102-125): per tet the
 * gradient of the P2 level set at its vertices, the mean of the end values on
 * its edges; every P2 node averages the values of all its tets, running mean
 * in tet order. */
void orc_grad_recovery(int64_t nt, const int32_t* tet_v, const int32_t* tet_e, const double* coords, int64_t nv,
                       int64_t ne, const double* ls_vert, const double* ls_edge, double* grad_vert, double* grad_edge) {
    double* cv = (double*)calloc((size_t)(nv + ne), sizeof(double));
    double* ce = cv + nv;
    for (int64_t i = 0; i < 3 * nv; ++i) grad_vert[i] = 0.;
    for (int64_t i = 0; i < 3 * ne; ++i) grad_edge[i] = 0.;
    for (int64_t t = 0; t < nt; ++t) {
        double xv[4][3], T[3][3], det, gl[4][3], f[10], gv[4][3];
        for (int i = 0; i < 4; ++i) memcpy(xv[i], coords + 3 * tet_v[4 * t + i], sizeof xv[i]);
        trafo(xv, T, &det);
        bary_grads(T, gl);
        gather_ls10(tet_v + 4 * t, tet_e + 6 * t, ls_vert, ls_edge, f);
        for (int i = 0; i < 4; ++i) {
            double b[4] = {0, 0, 0, 0}, g[10][3];
            b[i] = 1.;
            p2_grads(b, gl, g);
            for (int r = 0; r < 3; ++r) {
                double s = 0.;
                for (int k = 0; k < 10; ++k) s += f[k] * g[k][r];
                gv[i][r] = s;
            }
        }
        for (int i = 0; i < 10; ++i) {
            double val[3], *dst, *cnt;
            if (i < 4) {
                for (int r = 0; r < 3; ++r) val[r] = gv[i][r];
                dst = grad_vert + 3 * (int64_t)tet_v[4 * t + i];
                cnt = cv + tet_v[4 * t + i];
            } else {
                for (int r = 0; r < 3; ++r) val[r] = 0.5 * (gv[EV[i - 4][0]][r] + gv[EV[i - 4][1]][r]);
                dst = grad_edge + 3 * (int64_t)tet_e[6 * t + i - 4];
                cnt = ce + tet_e[6 * t + i - 4];
            }
            const double n = (*cnt += 1.);
            for (int r = 0; r < 3; ++r) dst[r] = ((n - 1.) / n) * dst[r] + (1. / n) * val[r];
        }
    }
    free(cv);
}

/* barycentric coordinates of the world point x with respect to tet t (they
 * may lie outside [0, 1]: the mapper extrapolates the tet's polynomials) */
static void qq_world2bary(const orc_qq_ctx* q, int64_t t, const double x[3], double b[4]) {
    double xv[4][3], T[3][3], det, gl[4][3];
    for (int i = 0; i < 4; ++i) memcpy(xv[i], q->coords + 3 * q->tet_v[4 * t + i], sizeof xv[i]);
    trafo(xv, T, &det);
    bary_grads(T, gl);
    double d[3] = {x[0] - xv[0][0], x[1] - xv[0][1], x[2] - xv[0][2]};
    b[0] = 1.;
    for (int k = 1; k < 4; ++k) {
        b[k] = dot3(gl[k], d);
        b[0] -= b[k];
    }
}

/* P2 level set, recovered gradient and the P2 basis gradients of tet t at b */
typedef struct {
    int64_t t;
    double gl[4][3], h, f[10], gh[10][3];
} qq_tet;
static void qq_set_tet(const orc_qq_ctx* q, int64_t t, qq_tet* c) {
    double xv[4][3], T[3][3], det;
    for (int i = 0; i < 4; ++i) memcpy(xv[i], q->coords + 3 * q->tet_v[4 * t + i], sizeof xv[i]);
    trafo(xv, T, &det);
    bary_grads(T, c->gl);
    c->h = cbrt(fabs(det));
    gather_ls10(q->tet_v + 4 * t, q->tet_e + 6 * t, q->ls_vert, q->ls_edge, c->f);
    for (int k = 0; k < 4; ++k) memcpy(c->gh[k], q->grad_vert + 3 * (int64_t)q->tet_v[4 * t + k], sizeof c->gh[k]);
    for (int k = 0; k < 6; ++k) memcpy(c->gh[4 + k], q->grad_edge + 3 * (int64_t)q->tet_e[6 * t + k], sizeof c->gh[k]);
    c->t = t;
}
static void qq_eval(const qq_tet* c, const double b[4], double* ls, double g_ls[3], double gh[3], double dgh[3][3]) {
    double phi[10], g[10][3];
    p2_vals(b, phi);
    p2_grads(b, c->gl, g);
    double l = 0.;
    for (int k = 0; k < 10; ++k) l += c->f[k] * phi[k];
    *ls = l;
    for (int r = 0; r < 3; ++r) {
        double s = 0., s2 = 0.;
        for (int k = 0; k < 10; ++k) {
            s += c->f[k] * g[k][r];
            s2 += c->gh[k][r] * phi[k];
        }
        g_ls[r] = s;
        gh[r] = s2;
    }
    if (dgh)
        for (int r = 0; r < 3; ++r)
            for (int s = 0; s < 3; ++s) {
                double v = 0.;
                for (int k = 0; k < 10; ++k) v += c->gh[k][r] * g[k][s];
                dgh[r][s] = v; /* sum_k gh_k (x) grad phi_k */
            }
}
/* solve the n x n system A x = b by Gaussian elimination with partial pivoting */
static int qq_solve(int n, double A[4][4], double b[4]) {
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i)
            if (fabs(A[i][k]) > fabs(A[p][k])) p = i;
        if (A[p][k] == 0.) return 0;
        if (p != k) {
            for (int j = 0; j < n; ++j) { double t = A[k][j]; A[k][j] = A[p][j]; A[p][j] = t; }
            double t = b[k]; b[k] = b[p]; b[p] = t;
        }
        for (int i = k + 1; i < n; ++i) {
            const double m = A[i][k] / A[k][k];
            for (int j = k; j < n; ++j) A[i][j] -= m * A[k][j];
            b[i] -= m * b[k];
        }
    }
    for (int k = n - 1; k >= 0; --k) {
        double s = b[k];
        for (int j = k + 1; j < n; ++j) s -= A[k][j] * b[j];
        b[k] = s / A[k][k];
    }
    return 1;
}

/* base point of the point b0 of tet t (QuaQuaMapperCL::base_point_newton,
 * levelset/levelsetmapper.cpp:551-566): Newton on F(x, s) = (x0 - x - s gh(x),
 * -ls(x)) with the Armijo backtracking of newton_solve (num/newton.h:70-113).
 * Every iterate is evaluated on tet t's own P2 level set and recovered
 * gradient, extended beyond the tet: in the reference, locate_new_point
 * (levelsetmapper.cpp:463-490) searches the neighbourhood only while its tet
 * argument is null, and QuaQuaMapperFunctionCL::set_point (:178-208) always
 * passes the current tet, so the base tet never changes.  Returns the tet and
 * barycentric coordinates of the base point, the quasi-distance dh and the
 * Newton iterations. */
static int qq_base_point(const orc_qq_ctx* q, int64_t t, const double b0[4], int64_t* bt, double bb[4], double* dh,
                         int* iters) {
    qq_tet c;
    qq_set_tet(q, t, &c);
    double x0[3];
    for (int r = 0; r < 3; ++r) {
        double s = 0.;
        for (int k = 0; k < 4; ++k) s += q->coords[3 * (int64_t)q->tet_v[4 * t + k] + r] * b0[k];
        x0[r] = s;
    }
    double x[4] = {x0[0], x0[1], x0[2], 0.}, b[4];
    memcpy(b, b0, sizeof b);
    double ls, g_ls[3], gh[3], dgh[3][3], F[4];
    qq_eval(&c, b, &ls, g_ls, gh, NULL);
    F[0] = F[1] = F[2] = 0.;
    F[3] = -ls;
    int iter;
    for (iter = 0;; ++iter) {
        const double normF = sqrt(F[0] * F[0] + F[1] * F[1] + F[2] * F[2] + F[3] * F[3]);
        if (iter >= q->maxiter || normF < q->tol) break;
        qq_eval(&c, b, &ls, g_ls, gh, dgh);
        double dF[4][4];
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) dF[i][j] = -x[3] * dgh[i][j];
            dF[i][i] -= 1.;
            dF[i][3] = -gh[i];
            dF[3][i] = -g_ls[i];
        }
        dF[3][3] = 0.;
        double A4[4][4], dx[4];
        memcpy(A4, dF, sizeof A4);
        memcpy(dx, F, sizeof dx);
        if (!qq_solve(4, A4, dx)) return ORC_ERR_BAD_INPUT;
        double Jdx[4] = {0, 0, 0, 0};
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) Jdx[i] += dF[i][j] * dx[j];
        const double slope = q->armijo * (F[0] * Jdx[0] + F[1] * Jdx[1] + F[2] * Jdx[2] + F[3] * Jdx[3]) / normF;
        double l = 0.5 * c.h / sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
        if (!(l < 1.)) l = 1.;
        int j, accepted = 0;
        double bn[4], Fn[4];
        for (j = 0; j < q->max_damping && l >= 1e-7; ++j, l *= 0.5) {
            double xn[4];
            for (int i = 0; i < 4; ++i) xn[i] = x[i] - l * dx[i];
            qq_world2bary(q, c.t, xn, bn);
            double lsn, gn[3], ghn[3];
            qq_eval(&c, bn, &lsn, gn, ghn, NULL);
            for (int i = 0; i < 3; ++i) Fn[i] = x0[i] - xn[i] - xn[3] * ghn[i];
            Fn[3] = -lsn;
            if (sqrt(Fn[0] * Fn[0] + Fn[1] * Fn[1] + Fn[2] * Fn[2] + Fn[3] * Fn[3]) < normF + slope * l) {
                accepted = 1;
                break;
            }
        }
        if (l < 1e-7) break;
        /* as newton_solve: without an accepted step the last halved factor is taken */
        for (int i = 0; i < 4; ++i) x[i] -= l * dx[i];
        if (!accepted) {
            qq_world2bary(q, c.t, x, bn);
            double lsn, gn[3], ghn[3];
            qq_eval(&c, bn, &lsn, gn, ghn, NULL);
            for (int i = 0; i < 3; ++i) Fn[i] = x0[i] - x[i] - x[3] * ghn[i];
            Fn[3] = -lsn;
        }
        memcpy(b, bn, sizeof b);
        memcpy(F, Fn, sizeof F);
    }
    qq_eval(&c, b, &ls, g_ls, gh, NULL);
    *dh = x[3] * norm3(gh);
    *bt = c.t;
    memcpy(bb, b, sizeof b);
    *iters = iter;
    return ORC_OK;
}

/* Jacobian of the mapping at the base point (QuaQuaMapperCL::jacobian,
 * levelset/levelsetmapper.cpp:590-638) and the unit normal n of the level set
 * there */
static void qq_jacobian(const orc_qq_ctx* q, int64_t bt, const double bb[4], double dh, double dph[3][3], double n[3]) {
    qq_tet c;
    qq_set_tet(q, bt, &c);
    double ls, g_ls[3], gh[3], dgh[3][3];
    qq_eval(&c, bb, &ls, g_ls, gh, dgh);
    const double ngh = norm3(gh), nn = norm3(g_ls);
    double qn[3];
    for (int r = 0; r < 3; ++r) {
        qn[r] = gh[r] / ngh;
        n[r] = g_ls[r] / nn;
    }
    double tq[3];  /* dgh^T q_n */
    for (int s = 0; s < 3; ++s) tq[s] = dgh[0][s] * qn[0] + dgh[1][s] * qn[1] + dgh[2][s] * qn[2];
    double dn[3][3], Q[3][3];
    const double qdn = dot3(qn, n);
    for (int r = 0; r < 3; ++r)
        for (int s = 0; s < 3; ++s) {
            dn[r][s] = (1. / ngh) * (dgh[r][s] - qn[r] * tq[s]);
            Q[r][s] = (r == s ? 1. : 0.) - (qn[r] / qdn) * n[s];
        }
    double B[3][3];  /* I + dh Q dn */
    for (int r = 0; r < 3; ++r)
        for (int s = 0; s < 3; ++s) {
            double v = 0.;
            for (int k = 0; k < 3; ++k) v += Q[r][k] * dn[k][s];
            B[r][s] = (r == s ? 1. : 0.) + dh * v;
        }
    for (int col = 0; col < 3; ++col) {
        double A4[4][4] = {{0}}, rhs[4] = {Q[0][col], Q[1][col], Q[2][col], 0.};
        for (int r = 0; r < 3; ++r)
            for (int s = 0; s < 3; ++s) A4[r][s] = B[r][s];
        qq_solve(3, A4, rhs);
        for (int r = 0; r < 3; ++r) dph[r][col] = rhs[r];
    }
}

int orc_qq_local(const orc_qq_ctx* q, int64_t t, double M[100], double A[100], double b[10], int* npts, int* newton) {
    init_quad();
    memset(M, 0, sizeof(double) * 100);
    memset(A, 0, sizeof(double) * 100);
    memset(b, 0, sizeof(double) * 10);
    *npts = 0;
    *newton = 0;
    double f10[10], ls4[4];
    gather_ls10(q->tet_v + 4 * t, q->tet_e + 6 * t, q->ls_vert, q->ls_edge, f10);
    memcpy(ls4, f10, sizeof ls4);
    int sg0 = sgn(ls4[0]), mixed = 0;
    for (int k = 1; k < 4; ++k) mixed |= sgn(ls4[k]) != sg0;
    if (!mixed) return ORC_OK; /* equalSigns on lattice 1: no patch */
    orc_patch_t P;
    int st = orc_make_patch1(ls4, &P);
    if (st) return st;
    if (P.n_facets == 0) return ORC_OK;
    double xv[4][3], T[3][3], det, gl[4][3];
    for (int i = 0; i < 4; ++i) memcpy(xv[i], q->coords + 3 * q->tet_v[4 * t + i], sizeof xv[i]);
    trafo(xv, T, &det);
    bary_grads(T, gl);
    /* the facets' world vertices; normal nl of facet 0 (SPatchCL::compute_normals) */
    double nl[3];
    {
        double w[3][3];
        for (int j = 0; j < 3; ++j)
            for (int c = 0; c < 3; ++c) {
                const double* bj = P.bary[P.facet[0][j]];
                w[j][c] = xv[0][c] * bj[0] + xv[1][c] * bj[1] + xv[2][c] * bj[2] + xv[3][c] * bj[3];
            }
        double u[3], v[3];
        for (int c = 0; c < 3; ++c) { u[c] = w[1][c] - w[0][c]; v[c] = w[2][c] - w[0][c]; }
        nl[0] = u[1] * v[2] - u[2] * v[1];
        nl[1] = u[2] * v[0] - u[0] * v[2];
        nl[2] = u[0] * v[1] - u[1] * v[0];
        const double nn = norm3(nl);
        for (int c = 0; c < 3; ++c) nl[c] /= nn;
    }
    for (int f = 0; f < P.n_facets; ++f) {
        double w[3][3];
        for (int j = 0; j < 3; ++j) {
            const double* bj = P.bary[P.facet[f][j]];
            for (int c = 0; c < 3; ++c) w[j][c] = xv[0][c] * bj[0] + xv[1][c] * bj[1] + xv[2][c] * bj[2] + xv[3][c] * bj[3];
        }
        double u[3], v[3], cr[3];
        for (int c = 0; c < 3; ++c) { u[c] = w[1][c] - w[0][c]; v[c] = w[2][c] - w[0][c]; }
        cr[0] = u[1] * v[2] - u[2] * v[1];
        cr[1] = u[2] * v[0] - u[0] * v[2];
        cr[2] = u[0] * v[1] - u[1] * v[0];
        const double fdet = norm3(cr) * (P.boundary[f] ? 0.5 : 1.0);
        /* orthonormal basis U of the facet plane (Gram-Schmidt of the edges) */
        double U[2][3];
        const double nu = norm3(u);
        for (int c = 0; c < 3; ++c) U[0][c] = u[c] / nu;
        const double vu = dot3(v, U[0]);
        double v2[3];
        for (int c = 0; c < 3; ++c) v2[c] = v[c] - vu * U[0][c];
        const double nv2 = norm3(v2);
        for (int c = 0; c < 3; ++c) U[1][c] = v2[c] / nv2;
        for (int qp = 0; qp < 7; ++qp) {
            double bq[4];
            for (int c = 0; c < 4; ++c)
                bq[c] = P.bary[P.facet[f][0]][c] * Q2D_NODE[qp][0] + P.bary[P.facet[f][1]][c] * Q2D_NODE[qp][1] +
                        P.bary[P.facet[f][2]][c] * Q2D_NODE[qp][2];
            const double wq = fdet * Q2D_W[qp];
            int64_t bt;
            double bb[4], dh;
            int it = 0;
            st = qq_base_point(q, t, bq, &bt, bb, &dh, &it);
            if (st) return st;
            *newton += it;
            ++*npts;
            double dph[3][3], n[3];
            qq_jacobian(q, bt, bb, dh, dph, n);
            /* surface measure: sqrt det Gram(dph U) (surfactant/ifacetransp.cpp:865-891) */
            double DU[2][3];
            for (int k = 0; k < 2; ++k)
                for (int r = 0; r < 3; ++r) DU[k][r] = dph[r][0] * U[k][0] + dph[r][1] * U[k][1] + dph[r][2] * U[k][2];
            const double g00 = dot3(DU[0], DU[0]), g01 = dot3(DU[0], DU[1]), g11 = dot3(DU[1], DU[1]);
            const double absd = sqrt(g00 * g11 - g01 * g01);
            /* W = dph^T + nl (n / (nl.n) - dph nl)^T (gradient_trafo, surfactant/ifacetransp.cpp:894-914), W^-1 */
            double dnl[3];
            for (int r = 0; r < 3; ++r) dnl[r] = dph[r][0] * nl[0] + dph[r][1] * nl[1] + dph[r][2] * nl[2];
            const double nln = dot3(nl, n);
            double W[3][3], Winv[3][3];
            for (int r = 0; r < 3; ++r)
                for (int s = 0; s < 3; ++s) W[r][s] = dph[s][r] + nl[r] * (n[s] / nln - dnl[s]);
            for (int col = 0; col < 3; ++col) {
                double A4[4][4] = {{0}}, rhs[4] = {col == 0, col == 1, col == 2, 0.};
                for (int r = 0; r < 3; ++r)
                    for (int s = 0; s < 3; ++s) A4[r][s] = W[r][s];
                qq_solve(3, A4, rhs);
                for (int r = 0; r < 3; ++r) Winv[r][col] = rhs[r];
            }
            double phi[10], g[10][3], sg[10][3];
            p2_vals(bq, phi);
            p2_grads(bq, gl, g);
            for (int i = 0; i < 10; ++i) {
                double tg[3];
                const double gn = dot3(g[i], nl);
                for (int r = 0; r < 3; ++r) tg[r] = g[i][r] - gn * nl[r];
                for (int r = 0; r < 3; ++r) sg[i][r] = Winv[r][0] * tg[0] + Winv[r][1] * tg[1] + Winv[r][2] * tg[2];
            }
            const double wa = wq * absd;
            for (int i = 0; i < 10; ++i)
                for (int j = 0; j < 10; ++j) {
                    M[i * 10 + j] += wa * phi[i] * phi[j];
                    A[i * 10 + j] += wa * dot3(sg[i], sg[j]);
                }
            /* load vector: f = c xyz at the base point */
            qq_tet cb;
            qq_set_tet(q, bt, &cb);
            double y[3];
            for (int r = 0; r < 3; ++r) {
                double s = 0.;
                for (int k = 0; k < 4; ++k) s += q->coords[3 * (int64_t)q->tet_v[4 * bt + k] + r] * bb[k];
                y[r] = s;
            }
            const double fy = q->rhs_c * y[0] * y[1] * y[2];
            for (int i = 0; i < 10; ++i) b[i] += wa * fy * phi[i];
        }
    }
    return ORC_OK;
}

/* one base point and the Jacobian there (test aid) */
int orc_qq_point(const orc_qq_ctx* q, int64_t t, const double b0[4], int64_t* bt, double bb[4], double* dh,
                 double dph[9], int* iters) {
    int st = qq_base_point(q, t, b0, bt, bb, dh, iters);
    if (st) return st;
    double J[3][3], n[3];
    qq_jacobian(q, *bt, bb, *dh, J, n);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) dph[3 * r + c] = J[r][c];
    return ORC_OK;
}
