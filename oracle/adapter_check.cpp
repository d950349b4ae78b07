// Checks of the DROPS drop-in shim (drops_gb300/adapter) against the reference
// -- TEST INFRASTRUCTURE, built by oracle/build_ref.sh where the reference
// sources exist.  It links the reference's own objects and libtracefem.
//
//   adapter_check flatten <n> <a> <out>
//       BrickBuilderCL [-a,a]^3 with n^3 cubes, P2 level set |x| - 1 by nodal
//       interpolation; writes the shim's Flatten / LevelSetValues arrays.
//   adapter_check gpu <n> <a>
//       Without a usable GPU: the shim must throw DROPSErrCL (no CPU
//       fallback); prints "no-gpu: <message>".  With a GPU: the shim's
//       DistributeDOFs, setupFESystem (M, A, C_n) and PCG against the
//       reference's own calls on the same objects; prints "gpu: ok" or fails.
#include <cmath>
#include <cstdio>
#include <iostream>
#include <string>

#include "geom/builder.h"
#include "misc/problem.h"
#include "num/krylovsolver.h"
#include "num/precond.h"
#include "surfactant/ifacetransp.h"
#include "tracefem_drops.h"

using namespace DROPS;

namespace {

void put(FILE* f, const std::string& name, char type, const void* data, uint64_t n, size_t es) {
    const uint32_t l = (uint32_t)name.size();
    std::fwrite(&l, 4, 1, f);
    std::fwrite(name.data(), 1, l, f);
    std::fwrite(&type, 1, 1, f);
    std::fwrite(&n, 8, 1, f);
    if (n) std::fwrite(data, es, n, f);
}

struct Problem {
    BrickBuilderCL brick;
    MultiGridCL mg;
    IdxDescCL lsIdx{P2_FE};
    VecDescCL ls;
    Problem(int n, double a)
        : brick(Point3DCL(-a), 2. * a * std_basis<3>(1), 2. * a * std_basis<3>(2), 2. * a * std_basis<3>(3), n, n, n),
          mg(brick) {
        lsIdx.DistributeDOFs(0, mg);
        ls.SetIdx(&lsIdx);
        const Uint li = lsIdx.GetIdx();
        DROPS_FOR_TRIANG_VERTEX(mg, 0, it) ls.Data[it->Unknowns(li)] = it->GetCoord().norm() - 1.;
        DROPS_FOR_TRIANG_EDGE(mg, 0, it)
            ls.Data[it->Unknowns(li)] = (0.5 * (it->GetVertex(0)->GetCoord() + it->GetVertex(1)->GetCoord())).norm() - 1.;
    }
};

int cmd_flatten(int n, double a, const char* out) {
    Problem p(n, a);
    const gpu::FlatLevel F = gpu::Flatten(p.mg, 0);
    std::vector<double> lv, le;
    gpu::LevelSetValues(p.mg, 0, p.ls, lv, le);
    FILE* f = std::fopen(out, "wb");
    if (!f) return 2;
    std::fwrite("TFG1", 1, 4, f);
    std::vector<int64_t> tv(F.tet_v.begin(), F.tet_v.end()), te(F.tet_e.begin(), F.tet_e.end()),
        ev(F.edge_v.begin(), F.edge_v.end());
    put(f, "coords", 'd', F.coords.data(), F.coords.size(), 8);
    put(f, "tet_v", 'l', tv.data(), tv.size(), 8);
    put(f, "tet_e", 'l', te.data(), te.size(), 8);
    put(f, "edge_v", 'l', ev.data(), ev.size(), 8);
    put(f, "ls_vert", 'd', lv.data(), lv.size(), 8);
    put(f, "ls_edge", 'd', le.data(), le.size(), 8);
    std::fclose(f);
    return 0;
}

double max_abs_diff(const MatrixCL& A, const MatrixCL& B) {
    if (A.num_rows() != B.num_rows() || A.num_nonzeros() != B.num_nonzeros()) return INFINITY;
    double d = 0.;
    for (size_t r = 0; r <= A.num_rows(); ++r)
        if (A.raw_row()[r] != B.raw_row()[r]) return INFINITY;
    for (size_t k = 0; k < A.num_nonzeros(); ++k) {
        if (A.raw_col()[k] != B.raw_col()[k]) return INFINITY;
        d = std::max(d, std::fabs(A.raw_val()[k] - B.raw_val()[k]));
    }
    return d;
}

int cmd_gpu(int n, double a) {
    Problem p(n, a);
    IdxDescCL ref(P1IF_FE), dev(P1IF_FE);
    size_t na_dev = 0;
    try {
        na_dev = gpu::DistributeDOFs(dev, 0, p.mg, &p.ls);
    } catch (DROPSErrCL const& e) {  // the shim has no CPU fallback
        std::cout << "no-gpu: ";
        e.what(std::cout) << std::endl;
        return 0;
    }
    const size_t na_ref = ref.DistributeDOFs(0, p.mg, &p.ls);
    if (na_ref != na_dev || ref.NumUnknowns() != dev.NumUnknowns()) {
        std::cout << "gpu: numbering differs" << std::endl;
        return 1;
    }
    DROPS_FOR_TRIANG_TETRA(p.mg, 0, it) {
        if (ref.Loc2Glo(*it) != dev.Loc2Glo(*it)) {
            std::cout << "gpu: Loc2Glo differs" << std::endl;
            return 1;
        }
    }
    MatrixCL mats[2][3];
    for (int side = 0; side < 2; ++side) {
        IdxDescCL* idx = side ? &dev : &ref;
        FESystem sys;
        sys.params.levelSet.SetIdx(&p.lsIdx);
        sys.params.levelSet.Data = p.ls.Data;
        FEMatDescCL M(idx, idx, &LocalAssembler::M_P1P1), A(idx, idx, &LocalAssembler::A_P1P1),
            C(idx, idx, &LocalAssembler::C_n_P1P1);
        sys.matrices = {&M, &A, &C};
        if (side) gpu::setupFESystem(p.mg, sys);
        else setupFESystem(p.mg, sys);
        mats[side][0] = M.Data;
        mats[side][1] = A.Data;
        mats[side][2] = C.Data;
    }
    for (int k = 0; k < 3; ++k) {
        double mx = 0.;
        for (size_t q = 0; q < mats[0][k].num_nonzeros(); ++q) mx = std::max(mx, std::fabs(mats[0][k].raw_val()[q]));
        if (!(max_abs_diff(mats[0][k], mats[1][k]) <= 1e-12 * mx)) {
            std::cout << "gpu: matrix " << k << " differs" << std::endl;
            return 1;
        }
    }
    MatrixCL S(1., mats[0][0], 1., mats[0][1], 2. * a / n, mats[0][2]);
    VectorCL b(1., S.num_rows()), x_ref(0., S.num_rows()), x_dev(0., S.num_rows());
    JACPcCL pc;
    PCGSolverCL<JACPcCL> solver(pc, 100000, 1e-10, true);
    solver.Solve(S, x_ref, b, ref.GetEx());
    gpu::PCGSolverCL gsolver(100000, 1e-10, true);
    if (!gsolver.Solve(S, x_dev, b, ref.GetEx())) {
        std::cout << "gpu: PCG did not converge" << std::endl;
        return 1;
    }
    const double rel = std::sqrt(dot(VectorCL(x_ref - x_dev), VectorCL(x_ref - x_dev)) / dot(x_ref, x_ref));
    if (!(rel <= 1e-9)) {
        std::cout << "gpu: PCG solution differs " << rel << std::endl;
        return 1;
    }
    std::cout << "gpu: ok" << std::endl;
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    try {
        const std::string cmd = argc > 1 ? argv[1] : "";
        if (cmd == "flatten" && argc == 5) return cmd_flatten(std::atoi(argv[2]), std::atof(argv[3]), argv[4]);
        if (cmd == "gpu" && argc == 4) return cmd_gpu(std::atoi(argv[2]), std::atof(argv[3]));
        std::cerr << "usage: adapter_check flatten <n> <a> <out> | gpu <n> <a>" << std::endl;
        return 2;
    } catch (DROPSErrCL const& e) {
        std::cout << "error: ";
        e.what(std::cout) << std::endl;
        return 1;
    } catch (std::exception const& e) {
        std::cout << "error: " << e.what() << std::endl;
        return 1;
    }
}
