/*
 * tracefem.h -- C ABI of the GB300 (sm_103a) TraceFEM path.
 *
 * Drop-in boundary for the TraceFEM surface-PDE path of DROPS: interface DOF
 * numbering, surface-patch quadrature assembly of the local forms into CSR
 * matrices, and the Jacobi-preconditioned PCG / GMRES solves.  Every entry
 * point takes plain pointers and sizes; all device memory is owned by the
 * context.  Host arrays passed in are copied; host arrays passed out are
 * filled by the call.  One context per host thread; calls on one context are
 * ordered on the context's stream and return after their results are ready.
 *
 * Numbering conventions (identical to the reference's):
 *   - tet local vertices 0..3, local edges 0..5 = (0,1),(0,2),(1,2),(0,3),(1,3),(2,3)
 *     (geom/topo.cpp VertOfEdgeAr);
 *   - a P2 level set is given by one value per vertex and one per edge
 *     (the P2 VecDescCL of the reference, split by simplex);
 *   - local DOF order of a P2 tet: 4 vertices, then 6 edges (IdxDescCL::Loc2Glo,
 *     misc/problem.h:314-331).
 *
 * Every function returns TF_OK (0) or one of the TF_ERR_* codes below; the
 * message of the last failure is available from tf_last_error().
 */
#ifndef TRACEFEM_H
#define TRACEFEM_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define TF_OK 0
#define TF_ERR_CUDA 1          /* a CUDA runtime call failed                                     */
#define TF_ERR_ZERO_NODE 2     /* level set exactly 0 at a node of a cut tet: distance() throws  */
                               /* std::invalid_argument (geom/subtriangulation.tpp:43-44)        */
#define TF_ERR_ZERO_PATTERN 3  /* all-zero sign pattern on a lattice sub-tet: RefPatchCL::instance */
                               /* throws DROPSErrCL (geom/reftetracut.h:152-153)                  */
#define TF_ERR_BAD_INPUT 4     /* null/inconsistent arguments, call out of order                 */
#define TF_ERR_NOT_CONVERGED 5 /* Krylov solve hit max_iter: the reference returns false         */
#define TF_ERR_CAPACITY 6      /* a fixed per-row / per-tet capacity was exceeded                */
#define TF_ERR_WATCHDOG 7      /* a device-side wait gave up (bounded spin); context stays usable */
#define TF_ERR_NO_DEVICE 8     /* no CUDA device, or the library was not built for it            */
#define TF_ERR_INTERNAL 9      /* an internal consistency check failed                          */

/* ---- finite elements, forms, level sets -------------------------------- */
#define TF_P1IF 1 /* P1IF_FE (misc/problem.h:73) */
#define TF_P2IF 2 /* P2IF_FE (misc/problem.h:75) */

/* matrix handles: the bilinear forms of LocalAssembler (surfactant/ifacetransp.h) */
#define TF_FORM_M 0      /* M_P1P1 :1568 / M_P2P2 :1579                                  */
#define TF_FORM_A 1      /* A_P1P1 :1522 / P2 surface-gradient Laplace-Beltrami           */
#define TF_FORM_CN 2     /* C_n_P1P1 :1545 / diagonal blocks of C_n_vecP2vecP2 :1458      */
#define TF_FORM_LAPM 3   /* LaplaceM_P1P1 :1533 (mobility chi(1-chi), cut off at 0)       */
#define TF_NUM_FORMS 4
#define TF_MAT_SYS 4     /* linear combination of forms (tf_lincomb), same pattern       */
#define TF_MAT_BLOCK 5   /* 2x2 Cahn-Hilliard block matrix (tf_ch_block), 2m rows        */
#define TF_MAT_USER 6    /* matrix uploaded with tf_matrix_upload                         */
#define TF_FORM_N 7      /* N_P1P1 :1590-1600 (wind convection, not symmetric; tf_wind_upload) */
#define TF_NUM_MATS 8

/* vector handles (device vectors owned by the context) */
#define TF_VEC_RHS 0 /* assembled load vector (F_concentration_P1 :1610 or its P2 analogue) */
#define TF_VEC_X 1
#define TF_VEC_B 2
#define TF_VEC_CHI 3 /* P1 concentration used by TF_FORM_LAPM                              */
#define TF_VEC_T0 4
#define TF_VEC_T1 5
#define TF_VEC_T2 6
#define TF_VEC_T3 7
#define TF_NUM_VECS 8

/* analytic level sets (surfactant/Surface.hpp) */
#define TF_LS_SPHERE 0    /* par: cx,cy,cz,r         phi = |x-c| - r            (Sphere::dist :71)  */
#define TF_LS_TORUS 1     /* par: R,r,axis           phi = |(rho-R, x_axis)| - r (Torus::dist :130)  */
#define TF_LS_ELLIPSOID 2 /* par: cx,cy,cz,a,b,c,Q[9] phi = |diag(1/a,1/b,1/c) Q^T (x-c)| - 1          */
#define TF_LS_PLANE 3     /* par: nx,ny,nz,d         phi = n.x - d                                   */

/* load-vector integrands f(x) for TF_VEC_RHS */
#define TF_RHS_NONE 0
#define TF_RHS_SPHERE_XYZ 1 /* par: cx,cy,cz,r,c: f = c*y0*y1*y2, y = ext(x) on the sphere (Surface::ext) */
#define TF_RHS_CONST 2      /* par: c */

#define TF_PREC_FP64 0  /* every Krylov operation in FP64                               */
#define TF_PREC_MIXED 1 /* FP32 inner Krylov iterations inside FP64 iterative refinement */

typedef struct tf_context tf_context;

/* ---- context ------------------------------------------------------------ */
/* Creates a context on CUDA device `device`.  Replaces nothing in the
 * reference (which has no device state); it owns all device memory.        */
int tf_create(tf_context** ctx, int device);
int tf_destroy(tf_context* ctx);
const char* tf_last_error(const tf_context* ctx);
const char* tf_status_string(int status);
/* The context's CUDA stream (a cudaStream_t), for callers that time or order
 * their own work against the library's.                                      */
void* tf_stream(tf_context* ctx);

/* ---- mesh: one triangulation level of MultiGridCL ------------------------- */
/* BrickBuilderCL(orig, e1, e2, e3, n1, n2, n3) (geom/builder.cpp:99-180): the
 * mesh is kept implicit on the device (vertex / tet / edge numbers follow from
 * the brick indices); vertex coordinates and tet order are the reference's,
 * bit for bit.  Edges are numbered by direction class, see tf_mesh_download. */
int tf_mesh_brick(tf_context* ctx, const double orig[3], const double e1[3], const double e2[3],
                  const double e3[3], int n1, int n2, int n3);
/* A general tetrahedral mesh given as flat arrays (what a MultiGridCL level
 * flattens to): coords[3*nv], tet_v[4*nt], tet_e[6*nt] (edge ids, local edge
 * order above), edge_v[2*ne].  Copied to the device.                         */
int tf_mesh_upload(tf_context* ctx, int64_t nv, const double* coords, int64_t nt, const int32_t* tet_v,
                   const int32_t* tet_e, int64_t ne, const int32_t* edge_v);
int tf_mesh_info(tf_context* ctx, int64_t* nv, int64_t* ne, int64_t* nt);
/* Materialises the mesh arrays on the host (any pointer may be NULL). */
int tf_mesh_download(tf_context* ctx, double* coords, int32_t* tet_v, int32_t* tet_e, int32_t* edge_v);

/* ---- narrow-band refinement: AdapTriangCL + DistMarkingStrategyCL --------- */
/* The surface driver's mesh step (surfphasesep/surfphasesep.cpp:170-181):
 * DistMarkingStrategyCL(dist, width, coarse_level, fine_level)
 * (levelset/marking_strategy.cpp:356-398) and AdapTriangCL::MakeInitialTriang
 * (levelset/adaptriang.cpp:36-44), i.e. at most 2 * fine_level rounds of
 * marking and MultiGridCL::Refine (geom/multigrid.cpp:389-453), with the
 * distance function of a TF_LS_SPHERE / TF_LS_TORUS / TF_LS_PLANE kind.
 * Runs on the device (level-synchronous passes; scans keep the reference's
 * list order).  The context's mesh is replaced by the last triangulation level
 * (TriangFillCL order, geom/multigrid.cpp:1072-1083) as an uploaded mesh:
 * tets, their vertex order and the coordinates are the reference's; vertices
 * and edges are numbered by first touch.  The level set and everything after
 * it must be set up again.  last_level, steps: may be NULL.
 * TF_ERR_BAD_INPUT also when the mesh's tets do not list their vertices in
 * one global order (BrickBuilderCL's do; the refinement relies on it).
 * The refinement's working memory comes from a device memory pool of the
 * context, kept for the next call and returned by tf_destroy.               */
int tf_mesh_refine_band(tf_context* ctx, int kind, const double* par, int npar, double width, int coarse_level,
                        int fine_level, int* last_level, int* steps);
/* The same refinement on host arrays, without a context or a device (the
 * reference's sequential steps on one core): a level-0 mesh (coords[3*nv],
 * tet_v[4*nt]) in, a handle to the refined mesh out.                          */
typedef struct tf_refined tf_refined;
int tf_refine_band(int64_t nv, const double* coords, int64_t nt, const int32_t* tet_v, int kind, const double* par,
                   int npar, double width, int coarse_level, int fine_level, tf_refined** out);
int tf_refined_info(const tf_refined* r, int64_t* nv, int64_t* ne, int64_t* nt, int* last_level, int* steps);
/* coords[3*nv], tet_v[4*nt], tet_e[6*nt], edge_v[2*ne], tet_level[nt],
 * tets_per_level[last_level+1] (the level lists of the multigrid, all tets
 * of each level); any pointer may be NULL.                                    */
int tf_refined_get(const tf_refined* r, double* coords, int32_t* tet_v, int32_t* tet_e, int32_t* edge_v,
                   int32_t* tet_level, int64_t* tets_per_level);
void tf_refined_free(tf_refined* r);
/* The 64 refinement rules the refinement uses (RefRuleCL / ChildDataCL,
 * geom/topo.h:185-223, geom/triang.cpp): nch[64] children per edge pattern,
 * children[64*8*4] their local points (vertex i < 4, midpoint of edge i - 4),
 * -1 past nch.  Either pointer may be NULL.                                   */
int tf_refine_rules(int32_t* nch, int32_t* children);

/* ---- level set: the P2 VecDescCL LocalAssemblerParams::levelSet ------------ */
/* Host values per vertex and per edge.  ls_edge == NULL gives the
 * P1-interpolated level set, edge = 0.5*(a+b) (LinearLSInit,
 * surfactant/surfactant.cpp:733-745).                                          */
int tf_levelset_upload(tf_context* ctx, const double* ls_vert, const double* ls_edge);
/* Analytic level set evaluated on the device at the vertices and, for p2 != 0,
 * at the edge midpoints 0.5*(x0+x1) (LSInit / VecDescCL::Interpolate); p2 == 0
 * gives edge = 0.5*(a+b).  Values equal the host evaluation bit for bit.       */
int tf_levelset_analytic(tf_context* ctx, int kind, const double* par, int npar, int p2);
int tf_levelset_download(tf_context* ctx, double* ls_vert, double* ls_edge);
/* The wind of N_P1P1 (TF_FORM_N): the vecP2IF field u_T of
 * LocalAssemblerParams::surfCahnHilliardParams (surfactant/ifacetransp.h:933,
 * buildWindCH :1129-1137), as interpolated by VecDescCL::Interpolate
 * (misc/problem.h:714-732): xyz at every mesh vertex (wind_vert[3 nv]) and at
 * every edge midpoint (wind_edge[3 ne], this library's edge numbering).      */
int tf_wind_upload(tf_context* ctx, const double* wind_vert, const double* wind_edge);

/* ---- interface DOFs -------------------------------------------------------- */
/* IdxDescCL::DistributeDOFs(level, mg, &levelSet, dist) (misc/problem.cpp:283-336):
 * a tet is active iff distance(its 10 level-set values) <= dist; DOFs are
 * numbered in first-touch order over active tets in triangulation order,
 * vertices 0..3 then (P2) edges 0..5.  Returns the number of active tets like
 * the reference; TF_ERR_ZERO_NODE where distance() throws.                    */
int tf_distribute_dofs(tf_context* ctx, int fe, double dist, int64_t* n_active, int64_t* n_dofs);
/* IdxDescCL::CreateNumbering for P1IF_FE -> CreateNumbOnInterfaceVertex
 * (misc/problem.cpp:443-505, legacy path): a vertex is a DOF iff the Quad2
 * integral of lambda_i^2 over the patch exceeds omit_bound*(6|T|)^(4/3).      */
int tf_create_numb_on_interface_p1(tf_context* ctx, double omit_bound, int64_t* n_active, int64_t* n_dofs);
/* dof_vert[nv], dof_edge[ne] (-1 = no DOF), active_tets[n_active], loc2glo[n_active*nloc]
 * (IdxDescCL::Loc2Glo per active tet); any pointer may be NULL.                 */
int tf_dofs_download(tf_context* ctx, int32_t* dof_vert, int32_t* dof_edge, int32_t* active_tets,
                     int32_t* loc2glo);
/* Length of the tet list tf_dofs_download returns (active tets; for the
 * legacy numbering every cut tet, which the legacy accumulators visit), the
 * number of DOFs and the FE type.                                             */
int tf_dofs_info(tf_context* ctx, int64_t* n_tets, int64_t* n_dofs, int* fe);
/* The legacy P1 surfactant system on the numbering of
 * tf_create_numb_on_interface_p1: SetupInterfaceMassP1 with
 * LocalInterfaceMassP1CL (surfactant/ifacetransp.h:881-906: Quad2_2D on the
 * lattice-2 patch, off-diagonal entries times alpha) into TF_MAT_M,
 * SetupLBP1 with LocalLaplaceBeltramiP1CL (:1657-1695: facet-normal tangential
 * gradients times D) into TF_MAT_A, and, when fpar != NULL,
 * SetupInterfaceRhsP1 (surfactant/ifacetransp.cpp:515-563: Quad5_2D on the
 * planar pieces of the 8 regular children) into TF_VEC_RHS with
 * f(x) = fpar[0] + fpar[1..3].x + fpar[4] x^2 + fpar[5] y^2 + fpar[6] z^2
 *        + fpar[7] xy + fpar[8] xz + fpar[9] yz.
 * The pattern holds the numbered pairs of every cut tet with a non-empty
 * patch (MatrixBuilderCL keeps explicit zeros).  TF_MAT_C / TF_MAT_LAPM are
 * left empty.  Returns TF_ERR_ZERO_PATTERN where the reference throws.       */
int tf_setup_interface_p1_legacy(tf_context* ctx, double alpha, double D, const double* fpar, int64_t* nnz);

/* Surface patches of the tets tets[0..count) (tet ids, host array) exactly as
 * SPatchCL<3>::make_patch<MergeCutPolicyCL> builds them from the level set
 * (geom/subtriangulation.tpp:191-228): per tet the facet count nf[count],
 * facets[count*16*3] (vertex numbers: edge cuts in discovery order, then the
 * copied zero vertices), boundary[count*16] (is_boundary_facet),
 * nverts[count] and verts[count*40*4] (barycentric coordinates).            */
int tf_patches_download(tf_context* ctx, const int32_t* tets, int64_t count, int32_t* nf, int32_t* facets,
                        int32_t* boundary, int32_t* nverts, double* verts);

/* ---- assembly ---------------------------------------------------------------- */
/* setupFESystem(mg, FESystem&) (surfactant/ifacetransp.cpp:566-622): for every
 * active tet, the patch of the level set on the order-2 principal lattice
 * (SPatchCL::make_patch<MergeCutPolicyCL>, geom/subtriangulation.tpp:191-228),
 * Quad5_2D on every facet (make_CompositeQuad5Domain2D, num/quadrature.tpp:265-332)
 * and Quad5 on the tet; the local forms of `forms` (bit mask over TF_FORM_*)
 * and, when rhs_kind != TF_RHS_NONE, the load vector into TF_VEC_RHS.  The CSR
 * pattern is the union of the active-tet blocks, rows sorted by column
 * (SparseMatBuilderCL::Build, num/spmat.h:620-678); values are summed in
 * triangulation order.  The pattern is kept and reused while the DOF
 * numbering is unchanged.                                                       */
int tf_setup_fe_system(tf_context* ctx, unsigned forms, int rhs_kind, const double* rhs_par, int npar,
                       int64_t* nnz);
/* Pattern and values of a matrix handle (rowptr[m+1] as size_t-compatible
 * int64, colind[nnz], vals[nnz]; any pointer may be NULL).                      */
int tf_matrix_info(tf_context* ctx, int mat, int64_t* rows, int64_t* nnz);
int tf_matrix_download(tf_context* ctx, int mat, int64_t* rowptr, int64_t* colind, double* vals);
/* A host CSR matrix (MatrixCL: size_t row/col, double values) as TF_MAT_USER. */
int tf_matrix_upload(tf_context* ctx, int64_t m, const int64_t* rowptr, const int64_t* colind,
                     const double* vals);
/* MatrixCL LinComb ctor (num/spmat.h:712-715) on the shared pattern:
 * TF_MAT_SYS = sum_k coeffs[k] * forms[k].                                      */
int tf_lincomb(tf_context* ctx, int nterms, const int* forms, const double* coeffs);
/* The Cahn-Hilliard block matrix of surfphasesep/surfphasesep.cpp:431-434 as
 * TF_MAT_BLOCK: [[alpha M (+ N), mob Amob + rho C], [eps2 A + beta M + eps2 rho C, -M]]
 * with A = TF_FORM_A (A_one); flags (bit mask): TF_CH_DEGENERATE_MOBILITY
 * takes Amob = TF_FORM_LAPM (A_deg) in the upper-right block, else A_one;
 * TF_CH_WIND adds TF_FORM_N to the upper-left block (the reference does so
 * when the wind is not zero, :419-420).                                      */
#define TF_CH_DEGENERATE_MOBILITY 1
#define TF_CH_WIND 2
int tf_ch_block(tf_context* ctx, double alpha, double mob, double rho, double eps2, double beta, int flags);
/* Mobility and wind of the time loops (tf_ch_steps, tf_ch_steps_learned,
 * tf_ch_steps_adaptive), the options of surfphasesep/surfphasesep.cpp:414-420:
 * TF_CH_DEGENERATE_MOBILITY assembles LaplaceM_P1P1 (mobility chi (1 - chi),
 * cut off at 0) from the current chi before every solve (chi_ext for the BDF2
 * solves) and uses it in the block; TF_CH_WIND adds N_P1P1 of the uploaded
 * wind (tf_wind_upload; constant in time) to the upper-left block.  0 (the
 * default): constant mobility, no wind.                                       */
int tf_ch_options(tf_context* ctx, int flags);

/* ---- vectors ----------------------------------------------------------------- */
int tf_vec_upload(tf_context* ctx, int vec, int64_t n, const double* host);
int tf_vec_download(tf_context* ctx, int vec, double* host, int64_t n);
int tf_vec_size(tf_context* ctx, int vec, int64_t* n);
/* VecDescBaseCL::Write(os, binary = true) (misc/problem.h:928-944): the count
 * as a 64-bit size_t, then the values as doubles, host byte order.           */
int tf_vec_write(tf_context* ctx, int vec, const char* path);
/* VecDescBaseCL::Read(is, binary = true) (misc/problem.h:947-975): a count
 * other than n_expected (n_expected >= 0) is TF_ERR_BAD_INPUT, where the
 * reference throws DROPSErrCL; n_expected < 0 takes the file's count.       */
int tf_vec_read(tf_context* ctx, int vec, const char* path, int64_t n_expected);
/* Sets vector `vec` to n copies of `value` on the device (e.g. a zero initial guess). */
int tf_vec_fill(tf_context* ctx, int vec, int64_t n, double value);
/* y = A x on device vectors (y_Ax, num/spmat.h:1684-1709). */
int tf_spmv(tf_context* ctx, int mat, int vec_x, int vec_y);
/* Kernel of tf_spmv (no reference counterpart; the solvers have their own).
 * TF_SPMV_KERNEL_FP64 (default): FP64 FMAs, a few ulps of sum |a_ij x_j|
 * per row.  TF_SPMV_KERNEL_PAIR: FP32-pair products (values stored as
 * row-scaled float pairs, x split per call), within 3e-13 of
 * sum |a_ij x_j| per row; a matrix with a value a pair cannot hold, or a
 * call whose x has a non-zero entry outside [2^-74, 2^100] or a non-finite
 * one, runs the FP64 FMAs.                                                    */
#define TF_SPMV_KERNEL_FP64 0
#define TF_SPMV_KERNEL_PAIR 1
int tf_spmv_options(tf_context* ctx, int kernel);
/* Arithmetic of the element forms in tf_setup_fe_system (no reference
 * counterpart).  TF_ASM_KERNEL_PAIR (default): per-tet geometry and the patch
 * in FP64, the quadrature points, the basis and the element sums in FP32-pair
 * arithmetic (~48 significant bits) for M, A, C_n (P1 and P2) and the constant
 * or TF_RHS_SPHERE_XYZ load vector.  TF_ASM_KERNEL_FP64: FP64 throughout.
 * LaplaceM_P1P1 and N_P1P1 always use FP64.                                    */
#define TF_ASM_KERNEL_PAIR 0
#define TF_ASM_KERNEL_FP64 1
int tf_assemble_options(tf_context* ctx, int kernel);

/* ---- solvers ------------------------------------------------------------------- */
/* PCGSolverCL<JACPcCL>(pc, max_iter, tol, rel).Solve(A, x, b) (num/krylovsolver.h:
 * 107-189, 1805-1836; Jacobi SolveGSstep<PB_JAC0>, num/precond.h:153-169):
 * x (vec_x) is the initial guess and the result; max_iter and tol are in/out
 * (used iterations / reached residual).  TF_PREC_MIXED runs FP32 PCG sweeps
 * inside FP64 iterative refinement with the same stopping test on the FP64
 * residual.  Returns TF_ERR_NOT_CONVERGED where the reference returns false.  */
int tf_pcg_jacobi(tf_context* ctx, int mat, int vec_b, int vec_x, int precision, int* max_iter, double* tol,
                  int rel);
/* FP64 kernel of tf_pcg_jacobi (TF_PREC_FP64).  No counterpart in the
 * reference, which has one PCG.  TF_PCG_FP64_CLASSIC (default) runs
 * PCGSolverCL's recurrences with two grid barriers per iteration (iteration
 * counts as the reference's).  TF_PCG_FP64_CG1 runs the single-barrier
 * Chronopoulos-Gear form of the mixed solver in FP64, with each block's share
 * of the system resident in shared memory where it fits (else the classic
 * kernel); it stops on the recursive residual and confirms convergence on the
 * true residual b - A x.                                                       */
#define TF_PCG_FP64_CLASSIC 0
#define TF_PCG_FP64_CG1 1
int tf_pcg_options(tf_context* ctx, int fp64_kernel);
/* Autotuned launch shapes.  No counterpart in the reference (its kernels are
 * OpenMP loops).  With tuning on (the default), the first tf_spmv / mixed
 * tf_pcg_jacobi on a matrix structure (rows, non-zeros, SELL slots) times the
 * candidate shapes on that matrix -- SpMV: 512 x {1, 2} and 256 x {2, 4}
 * threads x blocks per SM; mixed PCG: the shared-memory resident kernel, the
 * single-barrier kernel with 512 or with 256 threads per block -- on internal
 * scratch vectors and keeps the fastest for the context.  on = 0 keeps the
 * fixed defaults.  tf_autotune_info reports the choice for a matrix handle:
 * spmv_us[4] and pcg_us[3] (may be NULL) the measured microseconds per SpMV /
 * per PCG iteration of each candidate (for the PCG the slope between a 40- and
 * a 160-iteration run, launch and set-up excluded), pcg_kind 0 resident, 1 512
 * threads, 2 256 threads.                                                      */
int tf_autotune(tf_context* ctx, int on);
int tf_autotune_info(tf_context* ctx, int mat, int* spmv_threads, int* spmv_blocks_per_sm, int* pcg_kind,
                     float* spmv_us, float* pcg_us);
/* GMResSolverCL / GMRES (num/krylovsolver.h:320-463, 1924-1975): restarted
 * GMRES(restart) with modified Gram-Schmidt and Givens rotations, Jacobi
 * preconditioning of the diagonal (for TF_MAT_BLOCK: of both diagonal blocks),
 * method 0 = right, 1 = left preconditioning.                                 */
int tf_gmres_jacobi(tf_context* ctx, int mat, int vec_b, int vec_x, int restart, int method, int precision,
                    int* max_iter, double* tol, int rel);
/* Orthogonalisation of tf_gmres_jacobi in FP64: TF_ORTH_MGS (default) is the
 * reference's modified Gram-Schmidt, one grid barrier per projection;
 * TF_ORTH_CGS2 is classical Gram-Schmidt with one reorthogonalisation, three
 * grid barriers per Arnoldi step, right preconditioning only.  TF_PREC_MIXED
 * always uses CGS2 with FP32 Arnoldi cycles, each restart being one step of
 * FP64 iterative refinement (true residual and update of x in FP64).          */
#define TF_ORTH_MGS 0
#define TF_ORTH_CGS2 1
int tf_gmres_options(tf_context* ctx, int orth);

/* ---- batches of independent problems ----------------------------------------------- */
/* The reference solves one surface problem per MultiGridCL; these calls run
 * `count` independent problems of uneven size as one: instance i is the brick
 * n[3i..3i+2] cubes spanned by axes[9i..9i+8] (e1, e2, e3) from orig[3i..3i+2]
 * (BrickBuilderCL, geom/builder.cpp:99-180), numbered after instance i-1.
 * tf_distribute_dofs, tf_setup_fe_system and the per-form calls then work on
 * the whole batch: each instance gets exactly the DOF numbering, CSR rows and
 * entries it would get alone, shifted by the rows of the instances before it
 * (the matrices are block diagonal).                                           */
int tf_mesh_brick_batch(tf_context* ctx, int count, const int32_t* n, const double* orig, const double* axes);
/* Level set per instance: par holds count consecutive sets of npar values of
 * the TF_LS_* kind (LSInit / LinearLSInit, surfactant/surfactant.cpp:733-758). */
int tf_levelset_analytic_batch(tf_context* ctx, int kind, const double* par, int npar, int p2);
/* Per-instance ranges after tf_distribute_dofs (each array count+1 long, NULL
 * to skip): tets, cut (active) tets, rows (DOFs); nnz needs the pattern of
 * tf_setup_fe_system.                                                          */
int tf_batch_info(tf_context* ctx, int64_t* tets, int64_t* cut, int64_t* rows, int64_t* nnz);
/* TF_MAT_SYS = sum_k coeffs[i*nterms + k] * forms[k] on the rows of instance i
 * (the per-problem LinComb of num/spmat.h:712-715, e.g. M + A + h_i C_n).      */
int tf_batch_lincomb(tf_context* ctx, int nterms, const int* forms, const double* coeffs);
/* Jacobi-PCG (num/krylovsolver.h:107-189) on every instance at once, one
 * persistent launch: CTAs take instances from a queue, largest first, and
 * each solves its instance to relative residual tol (rel != 0) within
 * max_iter iterations, x (vec_x) being the initial guess and the result.
 * TF_PREC_MIXED: FP32 iterations with FP64 iterate and FP64 residual
 * replacement.  iters[count] and resids[count] (may be NULL) receive each
 * instance's iterations and reached residual; TF_ERR_NOT_CONVERGED when any
 * instance missed tol.  Unless tf_batch_config fixed them, the lanes per row
 * and CTA size come from tf_batch_tune, run on the first solve of a pattern,
 * and the launch sequence is captured once as a CUDA graph and replayed while
 * matrix, vectors and parameters stay the same.                                */
int tf_batch_pcg_jacobi(tf_context* ctx, int mat, int vec_b, int vec_x, int precision, int max_iter, double tol,
                        int rel, int* iters, double* resids);
/* Autotuner: times every (lanes per row in {2,4,8,16}, CTA size in
 * {128,256,512,1024}) candidate on this batch and keeps the fastest.           */
int tf_batch_tune(tf_context* ctx, int mat, int vec_b, int precision, int* lanes, int* threads);
/* lanes = 0: autotune; else fixed lanes per row and CTA size.  use_graph = 0
 * launches the solve directly instead of replaying a CUDA graph.               */
int tf_batch_config(tf_context* ctx, int lanes, int threads, int use_graph);

/* ---- learned warm start: per-DOF MLP on the tensor cores ------------------------- */
/* No counterpart in the reference (it starts each Cahn-Hilliard solve from the
 * previous state).  A per-DOF MLP, 80 BF16 inputs -> 64 -> 64 -> 64 -> 2 with
 * tanh, FP32 accumulation, run and trained by tcgen05 kernels.  Weights are
 * TF_MLP_WEIGHTS floats: four row-major [out][80] matrices (64, 64, 64 and 16
 * rows; the last layer's rows 2..15 are zero) whose bias is the column of the
 * constant-1 input (70 in the first layer, 64 in the others).  Inputs X are
 * n x 80 BF16 values (raw 16-bit patterns), targets and outputs n x 2 floats;
 * all buffers of these calls are host memory.                                  */
#define TF_MLP_IN 80
#define TF_MLP_WEIGHTS 16640
int tf_mlp_init(tf_context* ctx, uint64_t seed);
int tf_mlp_get_weights(tf_context* ctx, float* w);
int tf_mlp_set_weights(tf_context* ctx, const float* w);
int tf_mlp_forward(tf_context* ctx, const uint16_t* X, int64_t n, float* pred);
/* Gradient of the mean squared error over all n samples and both outputs,
 * weights unchanged; loss receives that mean.                                  */
int tf_mlp_gradient(tf_context* ctx, const uint16_t* X, const float* Y, int64_t n, float* grad, double* loss);
/* `epochs` passes of Adam (beta 0.9/0.999) over mini-batches of
 * minibatch_tiles x 128 samples; loss receives the last pass's mean error.     */
int tf_mlp_train(tf_context* ctx, const uint16_t* X, const float* Y, int64_t n, int epochs, int minibatch_tiles,
                 float lr, double* loss);
/* Inputs (and targets when vec_next >= 0) of every DOF for states cur = x_n
 * and old = x_{n-1} (vectors [chi; omega] of 2m values), as the learned
 * Cahn-Hilliard loop builds them; needs the P1 numbering and TF_FORM_M.       */
int tf_ch_features(tf_context* ctx, int vec_cur, int vec_old, int vec_next, uint16_t* X, float* Y);

/* ---- isoparametric P2 TraceFEM (QuaQua mapper) ------------------------------------ */
/* The P2 driver of surfactant/surfactant.cpp:1581-1640: InterfaceCommonDataP2CL
 * on PrincipalLatticeCL::instance(1) with QuaQuaMapperCL (Newton form,
 * levelset/levelsetmapper.cpp) and averaging_P2_gradient_recovery
 * (num/gradient_recovery.cpp:82), accumulating LocalMassP2CL,
 * LocalLaplaceBeltramiP2CL (D = 1) and LocalVectorP2CL with f(y) = f_coeff
 * y0 y1 y2 at the base points y (surfactant/ifacetransp.h:2286-2402).  Needs a
 * single brick mesh, a P2 level set and the P2IF numbering of tf_distribute_dofs;
 * writes the isoparametric mass matrix into TF_FORM_M, the Laplace-Beltrami
 * matrix into TF_FORM_A (on the DistributeDOFs pattern: entries of tets with
 * an empty linear interface are explicit zeros) and the load vector into
 * TF_VEC_RHS.  newton_tol / newton_maxiter: the mapper's Newton (the reference
 * driver reads them from LevelsetMapper.Tol / Iter); newton_iters_max (may be
 * NULL) receives the largest Newton count of a quadrature point.  As in the
 * reference, every base point is sought on its own tet's P2 level set and
 * recovered gradient, extended beyond the tet.                                   */
int tf_setup_quaqua_p2(tf_context* ctx, double f_coeff, double newton_tol, int newton_maxiter, int* newton_iters_max);

/* ---- allocation-free PCG -------------------------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory: applications that manage every GPU byte through their own pool and
 * forbid third-party cudaMalloc, real-time loops that must not pay the
 * implicit device synchronisation of cudaMalloc/cudaFree.  Jacobi-PCG as
 * tf_pcg_jacobi (FP64), but without a context: rowptr[m+1], colind[nnz]
 * (int32), vals[nnz], b[m] and x[m] (initial guess in, solution out) are
 * DEVICE pointers owned by the
 * caller; max_iter and tol are host in/out values as in tf_pcg_jacobi; stream
 * is a cudaStream_t or NULL.  All other memory the solve needs lives in one
 * fixed device array of the library (6*TF_NOALLOC_MAX_ROWS doubles plus a few
 * hundred KB, about 13 MB), which every GPU that loads the library holds until
 * the process exits.  The call allocates nothing.  m > TF_NOALLOC_MAX_ROWS
 * returns TF_ERR_CAPACITY.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) and should come before any stream
 * capture on that device.  Every call blocks the host: it reads nnz =
 * rowptr[m] back before the launch and waits on `stream` for the outcome.
 * Every call reuses
 * the same array: calls that overlap on the GPU (two streams, two host
 * threads) race on it and must be serialised by the caller.  Outcome as
 * tf_pcg_jacobi: TF_OK on convergence; TF_ERR_NOT_CONVERGED with *max_iter =
 * the iterations run and *tol = the true relative residual otherwise
 * (max_iter = 0 runs none and reports the initial residual).                  */
#define TF_NOALLOC_MAX_ROWS 262144
int tf_pcg_jacobi_noalloc(int64_t m, const int32_t* rowptr, const int32_t* colind, const double* vals,
                          const double* b, double* x, int* max_iter, double* tol, int rel, void* stream);

/* ---- Cahn-Hilliard time stepping ------------------------------------------------- */
/* `nsteps` implicit (BDF1) steps of the surface Cahn-Hilliard system of
 * surfphasesep/surfphasesep.cpp:397-440 (constant mobility, no wind):
 *   F_chi = f + (1/dt) M chi,  F_omega = beta_s M chi - M f0'(chi),
 *   f0'(c) = xi 2c(1-c)(1-2c) (surfphasesep.cpp:140-150),
 * block matrix [[M/dt (+ N), mob Amob + rho C], [eps^2 A + beta_s M + eps^2 rho C, -M]]
 * (TF_MAT_BLOCK), GMRES(restart) with nodal 2x2 block-Jacobi applied from the
 * right, relative residual tol.  Needs TF_FORM_M/A/CN assembled; f is
 * TF_VEC_RHS when it holds m values, else 0.  TF_VEC_X holds [chi; omega]
 * (2m) on entry and exit; warm != 0 starts every solve from the previous state
 * (the reference's UsePreviousFrameAsInitialGuess), warm == 0 from zero.
 * iters[nsteps], resids[nsteps] (may be NULL) receive each solve's GMRES
 * iteration count and relative residual; TF_VEC_CHI receives the final chi. */
int tf_ch_steps(tf_context* ctx, int nsteps, double dt, double mobility, double eps, double beta_s, double xi,
                double rho_vol, int restart, double tol, int max_iter, int warm, int* iters, double* resids);
/* Adaptive BDF1/BDF2 time stepping of surfphasesep/surfphasesep.cpp:397-483
 * (constant mobility, no wind).  Per step i, attempt after attempt:
 *   dt = F(e, dt) (first step, and every attempt when adaptive): dt0 for
 *        e == 0, else F_rho sqrt(F_tol / e) dt clamped to [F_min, F_max] (:117-123);
 *   BDF1 solve (alpha = 1/dt) from the state [chi; omega];
 *   BDF2 solve with r = dt/dt_prev, chi_ext = (1+r) chi - r chi_prev,
 *        F_chi = f + ((1+r)/dt) M chi - r^2/((1+r) dt) M chi_prev,
 *        F_omega = beta_s M chi_ext - M f0'(chi_ext), alpha = (1+2r)/((1+r) dt);
 *   e = sqrt(d'M d / chi2'M chi2), d = chi_BDF2 - chi_BDF1;
 * repeated while adaptive and e > F_tol and F_min < dt < F_max.  Step 1
 * takes the BDF1 solution.  The accepted state is the BDF2 solution
 * [chi; omega] in TF_VEC_X.  Solves: GMRES(restart) with nodal block Jacobi
 * (as tf_ch_steps), warm-started from the previous state.                   */
typedef struct {
    double t0, t_final, dt0;            /* start time, final time, Time.StepSize */
    double F_tol, F_rho, F_min, F_max;  /* step-size control */
    int adaptive, max_steps;            /* isTimeAdaptive, bound on accepted steps */
    double mobility, eps, beta_s, xi, rho_vol;
    int restart, max_iter;
    double tol;
} tf_ch_adapt_params;
/* nsteps: accepted steps; t_end: final time; per accepted step (arrays of
 * max_steps, may be NULL): dts, errs (e of the last attempt), tries, iters
 * (GMRES iterations of all its solves).                                      */
int tf_ch_steps_adaptive(tf_context* ctx, const tf_ch_adapt_params* p, int* nsteps, double* t_end, double* dts,
                         double* errs, int* tries, int* iters);
/* The integrals of the per-step statistics of surfphasesep/surfphasesep.cpp:
 * 324-345 (exportStats) for chi = TF_VEC_CHI, M = TF_FORM_M, A = TF_FORM_A,
 * f0(c) = xi (c (1 - c))^2 (:135-139): out[0] = 1'M1 (Integral.SurfacaAreaP1),
 * out[1] = 1'M chi / out[0] (RaftFraction), out[2] = eps chi'A chi
 * (PerimeterEstimate), out[3] = (M1)'f0(chi) + eps^2/2 chi'A chi
 * (LyapunovEnergy), out[4] / out[5] = max / min of chi (c_h.Max / c_h.Min). */
int tf_ch_stats(tf_context* ctx, double eps, double xi, double* out);
/* tf_ch_steps with the learned warm start: the MLP (tf_mlp_init first, or a
 * default initialisation) is trained online with `epochs` Adam passes
 * (minibatch_tiles x 128 DOFs, rate lr) on the increment of each of the first
 * train_steps steps.  The network predicts the deviation of the next state
 * from linear extrapolation.  learned = 1: the guess of a step is the
 * combination of the last 6 states (as backward differences) and, from the
 * network's third training step on, its predicted correction that minimises
 * the FP64 residual ||b - A x||; learned = 3: the same projection without the
 * network; learned = 2: linear extrapolation x_n + (x_n - x_{n-1});
 * learned = 0: the plain previous-state warm start of the reference.  A guess
 * is used when its FP64 residual is below the previous state's, and a step
 * whose guessed solve needed more than 5/4 of the GMRES iterations of the
 * last plain solve makes the next step use the previous state.  precision as
 * in tf_gmres_jacobi (the orthogonalisation of tf_gmres_options applies to
 * TF_PREC_FP64).  used[nsteps]
 * (may be NULL) flags the steps that started from the learned guess.          */
int tf_ch_steps_learned(tf_context* ctx, int nsteps, double dt, double mobility, double eps, double beta_s, double xi,
                        double rho_vol, int restart, double tol, int max_iter, int precision, int learned,
                        int train_steps, int epochs, int minibatch_tiles, float lr, int* iters, double* resids,
                        int* used);

/* ---- instrumentation -------------------------------------------------------------- */
/* Per-kernel device time, recorded with CUDA events on the context's stream
 * while enabled; kernel ids are the TF_K_* below.                                  */
#define TF_K_CLASSIFY 0
#define TF_K_NUMBER 1
#define TF_K_ASSEMBLE 2
#define TF_K_PATTERN 3
#define TF_K_SCATTER 4
#define TF_K_SPMV 5
#define TF_K_PCG 6
#define TF_K_GMRES 7
#define TF_K_LEVELSET 8
#define TF_K_BATCH 9
#define TF_NUM_KERNELS 10
int tf_timing_enable(tf_context* ctx, int on);
int tf_timing_get(tf_context* ctx, int kernel, double* total_ms, int64_t* launches);
int tf_timing_reset(tf_context* ctx);
/* number of kernels this library launched on the context since creation */
int64_t tf_launch_count(tf_context* ctx);
/* CUDA events on the context's stream: record marker `slot` (0..7) and read
 * the elapsed device time between two recorded markers.                     */
int tf_marker_record(tf_context* ctx, int slot);
int tf_marker_elapsed(tf_context* ctx, int slot_a, int slot_b, double* ms);
/* Measurement helper (no reference counterpart): `reps` calls of tf_spmv,
 * each bracketed by CUDA events on the context's stream and preceded by an L2
 * flush when `cold` is 1 (twice the L2 size written: dirty lines left behind)
 * or 2 (twice the L2 size read: L2 left clean); the launches are queued
 * without host waits so the events time the kernel alone.  ms_each[r] =
 * device time of call r.                                                      */
int tf_spmv_timed(tf_context* ctx, int mat, int vec_x, int vec_y, int reps, int cold, float* ms_each);
/* Measurement helper (no reference counterpart): the streaming floor for a
 * transfer size.  `reps` launches of a coalesced read of `bytes` bytes, timed
 * like tf_spmv_timed (flush, event, kernel, event queued back to back).      */
int tf_stream_read_timed(tf_context* ctx, int64_t bytes, int reps, int cold, float* ms_each);
/* Overwrites a scratch buffer of twice the L2 size on the context's stream,
 * so that the next call starts with a cold L2.                               */
int tf_flush_l2(tf_context* ctx);
/* Page-locked host memory for callers that stage inputs/outputs (NULL on failure). */
void* tf_host_alloc(size_t bytes);
void tf_host_free(void* p);

#ifdef __cplusplus
}
#endif
#endif
