// Drop-in GPU versions of the DROPS TraceFEM calls, for code that links DROPS.
//
// These functions keep the reference's call surface and its data types
// (MultiGridCL, IdxDescCL, FESystem, MatrixCL, VectorCL) and do the work
// through libtracefem's C ABI (include/tracefem.h) on the GPU:
//
//   DROPS::gpu::DistributeDOFs(idx, level, mg, &levelSet, dist)
//       for IdxDescCL::DistributeDOFs (misc/problem.cpp:283-336)
//   DROPS::gpu::setupFESystem(mg, system)
//       for setupFESystem (surfactant/ifacetransp.cpp:615-622)
//   DROPS::gpu::PCGSolverCL(maxiter, tol, rel).Solve(A, x, b, ex)
//       for PCGSolverCL<JACPcCL> (num/krylovsolver.h:1805-1836)
//   DROPS::gpu::GMResSolverCL(restart, maxiter, tol, rel).Solve(A, x, b, ex)
//       for GMResSolverCL<JACPcCL> (num/krylovsolver.h:1924-1975), right
//       preconditioning
//
// A triangulation level is flattened once (vertex, edge and tet order of the
// triangulation; tet-local vertex / edge order of geom/topo.cpp) and uploaded
// as an explicit mesh; it is uploaded again when the level's vertex, edge or
// tet count changes or after Invalidate().  The numbering that
// DistributeDOFs computes on the GPU is written back into the UnknownHandleCLs,
// so Loc2Glo, output and the reference's own routines see the reference's
// numbering.  Matrices come back as MatrixCL (size_t CSR, rows sorted by
// column, explicit zeros kept, as SparseMatBuilderCL::Build).
//
// Errors follow the reference: an exact zero of the level set at a node of a
// cut tet throws std::invalid_argument (distance(),
// geom/subtriangulation.tpp:43-44); an all-zero sign pattern and every other
// failure throw DROPSErrCL; non-convergence is returned as false.  There is
// no CPU fallback: without a usable GPU every call throws.
//
// Supported forms: M_P1P1, A_P1P1, C_n_P1P1, LaplaceM_P1P1 (degenerate
// mobility from params.surfCahnHilliardParams.chi), N_P1P1 (wind from
// params.surfCahnHilliardParams.u_T, a vecP2IF vector), M_P2P2.  The load
// vector F_concentration_P1 needs a right-hand side the GPU can evaluate:
// SetLoad(kind, parameters) with a TF_RHS_* kind (an arbitrary host function
// cannot run on the device).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "misc/problem.h"
#include "surfactant/ifacetransp.h"
#include "tracefem.h"

namespace DROPS {
namespace gpu {

// The calling thread's libtracefem context on CUDA device 0 (created on first
// use; throws DROPSErrCL when there is no usable sm_103a GPU).
tf_context* context();

// Forget the uploaded mesh and level set (the next call uploads them again).
void Invalidate();

// Load vector of setupFESystem: a TF_RHS_* kind and its parameters.
void SetLoad(int rhs_kind, const std::vector<double>& parameters);

// A triangulation level in flat arrays (the C ABI's explicit mesh).
struct FlatLevel {
    std::vector<double> coords;   // 3 per vertex
    std::vector<int32_t> tet_v;   // 4 per tet (VertexCL order of the tet)
    std::vector<int32_t> tet_e;   // 6 per tet (EdgeCL order of the tet)
    std::vector<int32_t> edge_v;  // 2 per edge
};
FlatLevel Flatten(const MultiGridCL& mg, Uint level);
// P2 level-set values at the flattened vertices and edges
void LevelSetValues(const MultiGridCL& mg, Uint level, const VecDescCL& ls, std::vector<double>& ls_vert,
                    std::vector<double>& ls_edge);

size_t DistributeDOFs(IdxDescCL& idx, Uint level, MultiGridCL& mg, VecDescCL const* levelSet, double dist = 0.);

void setupFESystem(MultiGridCL const& mg, FESystem& system);

class PCGSolverCL {
  public:
    PCGSolverCL(int maxiter, double tol, bool rel = false, int precision = TF_PREC_FP64)
        : maxiter_(maxiter), tol_(tol), rel_(rel), precision_(precision) {}
    template <typename ExT>
    bool Solve(const MatrixCL& A, VectorCL& x, const VectorCL& b, const ExT&) {
        return solve(A, x, b);
    }
    int GetIter() const { return iter_; }
    double GetResid() const { return res_; }

  private:
    bool solve(const MatrixCL& A, VectorCL& x, const VectorCL& b);
    int maxiter_;
    double tol_;
    bool rel_;
    int precision_;
    int iter_ = -1;
    double res_ = -1.;
};

class GMResSolverCL {
  public:
    GMResSolverCL(int restart, int maxiter, double tol, bool rel = true, int precision = TF_PREC_FP64)
        : restart_(restart), maxiter_(maxiter), tol_(tol), rel_(rel), precision_(precision) {}
    template <typename ExT>
    bool Solve(const MatrixCL& A, VectorCL& x, const VectorCL& b, const ExT&) {
        return solve(A, x, b);
    }
    int GetIter() const { return iter_; }
    double GetResid() const { return res_; }

  private:
    bool solve(const MatrixCL& A, VectorCL& x, const VectorCL& b);
    int restart_, maxiter_;
    double tol_;
    bool rel_;
    int precision_;
    int iter_ = -1;
    double res_ = -1.;
};

}  // namespace gpu
}  // namespace DROPS
