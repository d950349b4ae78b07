/*
 * CPU oracle for the TraceFEM hot path of DROPS.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm, used by tests/ as the checker, by __graft_entry__.smoke() as the
 * checker, and by bench.py as the timed CPU baseline ("port").  The product
 * path (drops_gb300/, include/tracefem.h) never links, loads or calls it.
 *
 * Each function names the reference file:line it restates (paths relative to
 * the DROPS source tree, src/).  Parity of this restatement is pinned against
 * the reference itself: oracle/build_ref.sh compiles the reference's own
 * sources into oracle/_ref/ref_harness, tests/golden/make_golden.py runs it
 * and stores its outputs as fixtures, and tests/test_oracle_golden.py checks
 * this file against those fixtures.
 */
#ifndef TRACEFEM_ORACLE_H
#define TRACEFEM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (same meaning as include/tracefem.h) */
#define ORC_OK 0
#define ORC_ERR_ZERO_NODE 2    /* level set exactly zero at a node of a cut tet */
#define ORC_ERR_ZERO_PATTERN 3 /* all four lattice values of a sub-tet are zero */
#define ORC_ERR_BAD_INPUT 4
#define ORC_ERR_NOT_CONVERGED 5
#define ORC_ERR_CAPACITY 6

/* ---- mesh: BrickBuilderCL (geom/builder.cpp:99-180) ------------------- */
int64_t orc_brick_num_vertices(int n1, int n2, int n3);
int64_t orc_brick_num_edges(int n1, int n2, int n3);
int64_t orc_brick_num_tets(int n1, int n2, int n3);
/* coords[3*nv], tet_v[4*nt], tet_e[6*nt], edge_v[2*ne] */
void orc_brick(const double orig[3], const double e1[3], const double e2[3], const double e3[3],
               int n1, int n2, int n3, double* coords, int32_t* tet_v, int32_t* tet_e, int32_t* edge_v);

/* ---- level sets (surfactant/Surface.hpp, surfactant/surfactant.cpp:733-758) */
#define ORC_LS_SPHERE 0    /* par: cx, cy, cz, r                         */
#define ORC_LS_TORUS 1     /* par: R, r, axis                            */
#define ORC_LS_ELLIPSOID 2 /* par: cx,cy,cz, a,b,c, R[9] (row-major)     */
#define ORC_LS_PLANE 3     /* par: nx,ny,nz, d  -> n.x - d               */
double orc_ls_value(int kind, const double* par, const double x[3]);
/* vertex values, then edge values; p2 = 0: edge = 0.5*(a+b) (LinearLSInit),
 * p2 = 1: edge = phi(0.5*(x0+x1)) (LSInit / VecDescCL::Interpolate).      */
void orc_levelset(int kind, const double* par, int p2, int64_t nv, int64_t ne, const double* coords,
                  const int32_t* edge_v, double* ls_vert, double* ls_edge);

/* ---- DOF numbering: IdxDescCL::DistributeDOFs (misc/problem.cpp:283-336) */
/* dof_vert[nv], dof_edge[ne] (may be NULL when p2 == 0), active[nt] (0/1).
 * Returns ORC_ERR_ZERO_NODE like distance() throws
 * (geom/subtriangulation.tpp:38-46).                                       */
int orc_distribute_dofs(int64_t nt, const int32_t* tet_v, const int32_t* tet_e, int64_t nv, int64_t ne,
                        const double* ls_vert, const double* ls_edge, int p2, double dist,
                        int64_t* n_active, int64_t* n_dofs, int32_t* dof_vert, int32_t* dof_edge,
                        uint8_t* active);

/* Legacy numbering: CreateNumbOnInterfaceVertex (misc/problem.cpp:443-505). */
int orc_numb_on_interface_p1(int64_t nt, const int32_t* tet_v, const int32_t* tet_e, int64_t nv,
                             const double* coords, const double* ls_vert, const double* ls_edge,
                             double omit_bound, int64_t* n_active, int64_t* n_dofs, int32_t* dof_vert);

/* ---- surface patch on the lattice of order 2 --------------------------- */
#define ORC_MAX_FACETS 16
#define ORC_MAX_PVERTS 40
typedef struct {
    int n_facets, n_verts, n_cut_verts;
    int facet[ORC_MAX_FACETS][3];
    int boundary[ORC_MAX_FACETS];
    double bary[ORC_MAX_PVERTS][4];
} orc_patch_t;
/* SPatchCL<3>::make_patch<MergeCutPolicyCL> (geom/subtriangulation.tpp:191-228)
 * ls10: level set in P2 local order (4 vertices, 6 edges).                */
int orc_make_patch(const double ls10[10], orc_patch_t* p);
/* the same on PrincipalLatticeCL::instance(1) (the tet itself); ls4 at its vertices */
int orc_make_patch1(const double ls4[4], orc_patch_t* p);
void orc_lattice2(double verts[10][4], int tets[8][4]);

/* ---- assembly: setupFESystem (surfactant/ifacetransp.cpp:566-622) ------ */
#define ORC_FORM_M 0        /* M_P1P1 / M_P2P2                                    */
#define ORC_FORM_A 1        /* A_P1P1 / A_P2P2 (Laplace-Beltrami)                 */
#define ORC_FORM_CN 2       /* C_n_P1P1 / C_n_P2P2 (normal-gradient volume stab.) */
#define ORC_FORM_LAPM 3     /* LaplaceM_P1P1 (degenerate mobility)                */
#define ORC_FORM_N 4        /* N_P1P1 (wind convection, not symmetric; P1 only)   */
#define ORC_NUM_MAT_FORMS 5
#define ORC_RHS_NONE 0
#define ORC_RHS_SPHERE_XYZ 1 /* f(y) = c*y0*y1*y2 at y = ext(x) of a sphere (par: cx,cy,cz,r,c) */
#define ORC_RHS_CONST 2      /* f = c                                                          */

typedef struct {
    int p2;                /* 0: P1 forms, 1: P2 forms */
    unsigned forms;        /* bit mask over ORC_FORM_* */
    int rhs_kind;          /* ORC_RHS_*                */
    double rhs_par[8];
    const double* chi;     /* P1 vector (per DOF) for LaplaceM; NULL -> mobility 1 */
    int degenerate;        /* LaplaceM uses chi(1-chi) clipped at 0 when set        */
    const double* wind_vert; /* N: P2 wind, xyz per mesh vertex (3 nv)              */
    const double* wind_edge; /* N: xyz per mesh edge, at its midpoint (3 ne)        */
} orc_assemble_opts;

/* Builds the CSR pattern (union of active-tet blocks, rows sorted) and the
 * values of each requested matrix form plus the rhs vector.  rowptr[m+1] is
 * filled, colind/vals are allocated with malloc (caller frees with free()).
 * vals[f] stays NULL for forms not requested.                             */
int orc_assemble(int64_t nt, const int32_t* tet_v, const int32_t* tet_e, const double* coords,
                 const double* ls_vert, const double* ls_edge, const uint8_t* active,
                 const int32_t* dof_vert, const int32_t* dof_edge, int64_t m,
                 const orc_assemble_opts* opts, int64_t* rowptr, int32_t** colind, int64_t* nnz,
                 double* vals[ORC_NUM_MAT_FORMS], double* rhs);

/* local element matrices of one tet (nloc = 4 or 10) for tests */
int orc_local_forms(const double xv[4][3], const double ls10[10], const orc_assemble_opts* opts,
                    const double* chi_loc, const double* wind_loc, double out[ORC_NUM_MAT_FORMS][100],
                    double rhs[10], int* n_facets);

/* ---- legacy P1 interface forms (surfactant.cpp path) ------------------- */
/* f(x) = p0 + p1 x + p2 y + p3 z + p4 x^2 + p5 y^2 + p6 z^2 + p7 xy + p8 xz + p9 yz */
double orc_rhs_quadratic(const double* p, const double x[3]);
/* planar pieces of regular child ch (InterfaceTriangleCL::ComputeForChild) */
int orc_legacy_child_triangles(const double xv[4][3], const double ls10[10], int ch, double tri[2][3][4],
                               double det[2]);
/* LocalInterfaceMassP1CL (alpha), LocalLaplaceBeltramiP1CL (D), and the tet's
 * SetupInterfaceRhsP1 contributions; nonempty = lattice patch has facets     */
int orc_legacy_local(const double xv[4][3], const double ls10[10], double alpha, double D, const double* fpar,
                     double mass[16], double lb[16], double rhs[4], int* nonempty);
/* SetupInterfaceMassP1 / SetupLBP1 / SetupInterfaceRhsP1 over a mesh with a P1
 * numbering (dof_vert, -1 = not numbered); CSR and values malloc'ed.         */
int orc_assemble_legacy_p1(int64_t nt, const int32_t* tet_v, const int32_t* tet_e, const double* coords,
                           const double* ls_vert, const double* ls_edge, const int32_t* dof_vert, int64_t m,
                           double alpha, double D, const double* fpar, int64_t* rowptr, int32_t** colind,
                           int64_t* nnz, double** mass, double** lb, double* rhs);

/* ---- sparse linear algebra and solvers --------------------------------- */
void orc_spmv(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* vals,
              const double* x, double* y);
double orc_kahan_dot(int64_t n, const double* x, const double* y);
/* PCG with JACPcCL (num/krylovsolver.h:107-189, num/precond.h:153-169) */
int orc_pcg_jacobi(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* vals,
                   const double* b, double* x, int* max_iter, double* tol, int rel);
/* GMRES (num/krylovsolver.h:320-463), Jacobi preconditioner, left (method=1)
 * or right (method=0) preconditioning.                                      */
int orc_gmres_jacobi(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* vals,
                     const double* b, double* x, int restart, int* max_iter, double* tol, int rel,
                     int method);
/* block != 0: nodal 2x2 block Jacobi on a 2x2 block system (rows i and i+m/2) */
int orc_gmres(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* vals, const double* b,
              double* x, int restart, int* max_iter, double* tol, int rel, int method, int block);

/* Cahn-Hilliard 2x2 block system (surfphasesep/surfphasesep.cpp:431-434):
 * [[a*M, mob*A + rho*C], [eps2*A + beta*M + eps2*rho*C, -M]] with the shared
 * pattern of M/A/C.  Output pattern has 2m rows.                            */
int orc_ch_block(int64_t m, const int64_t* rowptr, const int32_t* colind, const double* M, const double* A,
                 const double* C, const double* Amob, const double* N, double alpha, double mob, double rho,
                 double eps2, double beta, int64_t* browptr, int32_t* bcolind, double* bvals);

/* 2 threads per call unless set; 1 means serial. */
void orc_set_threads(int n);

#ifdef __cplusplus
}
#endif

/* ---- isoparametric P2 TraceFEM (QuaQua mapper) ----------------------------- */
/* averaging_P2_gradient_recovery (num/gradient_recovery.cpp:82-89): grad_vert[3 nv], grad_edge[3 ne] */
void orc_grad_recovery(int64_t nt, const int32_t* tet_v, const int32_t* tet_e, const double* coords, int64_t nv,
                       int64_t ne, const double* ls_vert, const double* ls_edge, double* grad_vert, double* grad_edge);
typedef struct {
    const double* coords;
    const int32_t* tet_v;
    const int32_t* tet_e;
    const double* ls_vert;   /* P2 level set */
    const double* ls_edge;
    const double* grad_vert; /* recovered gradient */
    const double* grad_edge;
    double tol, armijo;      /* Newton of the mapper */
    int maxiter, max_damping;
    double rhs_c;            /* load f = rhs_c x y z at the base points */
} orc_qq_ctx;
/* LocalMassP2CL, LocalLaplaceBeltramiP2CL (D = 1) and LocalVectorP2CL of tet t
 * (surfactant/ifacetransp.h:2286-2402): full 10x10 M, A (row-major), b[10];
 * npts quadrature points, newton the Newton iterations of their base points */
int orc_qq_local(const orc_qq_ctx* q, int64_t t, double M[100], double A[100], double b[10], int* npts, int* newton);
/* one base point of tet t's point b0 (barycentric), its quasi-distance and the Jacobian of the mapping there */
int orc_qq_point(const orc_qq_ctx* q, int64_t t, const double b0[4], int64_t* bt, double bb[4], double* dh,
                 double dph[9], int* iters);

#endif
