// Harness around the DROPS reference implementation -- TEST INFRASTRUCTURE.
//
// Compiled by oracle/build_ref.sh against the reference's own sources (read
// in place, never copied) into oracle/_ref/ref_harness.  It drives the
// reference's public API for the TraceFEM path and writes what it computes
// to a small binary file (named arrays) that tests/golden/make_golden.py turns
// into committed fixtures.  Nothing here is shipped or timed as the product.
//
//   ref_harness system  <p1|p2> <lsP1|lsP2> <shape> <n> <a> <solve:0|1> <out>
//       BrickBuilderCL [-a,a]^3 with n^3 cubes (geom/builder.cpp:99-180),
//       P2 level-set index via DistributeDOFs (surfphasesep.cpp:184-190),
//       interface index DistributeDOFs (misc/problem.cpp:283-336),
//       setupFESystem (surfactant/ifacetransp.cpp:615-622) for M, A, C_n (+F),
//       optional PCGSolverCL<JACPcCL> on M + A + h C_n (num/krylovsolver.h:1805).
//   ref_harness system_ref <p1|p2> <lsP1|lsP2> <shape> <n> <a> <solve> <width> <coarse> <fine> <out>
//       the same on the last level after narrow-band refinement of the brick
//       (solve -1: the mesh only)
//       (AdapTriangCL::MakeInitialTriang with DistMarkingStrategyCL,
//       surfphasesep/surfphasesep.cpp:170-181; levelset/adaptriang.cpp,
//       levelset/marking_strategy.cpp:356-398, geom/multigrid.cpp:389-453).
//   ref_harness rules <out>                 the 64 refinement rules (geom/topo.cpp)
//   ref_harness legacy_numb <case> <out>    CreateNumbOnInterface test cases
//   ref_harness legacy_forms <n> <a> <out>  SetupInterfaceMassP1 / SetupLBP1 / SetupInterfaceRhsP1
//       (surfactant/ifacetransp.cpp:367-380, 499-512, 532-563) on the unit sphere,
//       P2 level set, CreateNumbering(P1IF_FE)
//   ref_harness area <out>                  tests/principallattice.cpp:316-347
//   ref_harness gmres_ref <n> <a> <steps> <width> <coarse> <fine> <out>
//       the same on the last level of the brick refined towards the torus
//       (AdapTriangCL::MakeInitialTriang, DistMarkingStrategyCL).
//   ref_harness quaqua <n> <a> <out>
//       Isoparametric P2 TraceFEM on the unit sphere (surfactant/surfactant.cpp:
//       1581-1640): P2 level set by nodal interpolation, the recovered
//       gradient (averaging_P2_gradient_recovery, num/gradient_recovery.cpp:82),
//       the QuaQua mapper (levelset/levelsetmapper.cpp, Newton form) and
//       LocalMassP2CL / LocalLaplaceBeltramiP2CL / LocalVectorP2CL
//       (surfactant/ifacetransp.h:2286-2402) on the linear interface
//       (principal lattice 1), accumulated on the DistributeDOFs P2IF numbering.
//   ref_harness gmres <n> <a> <steps> <out>
//       Torus (R = 1, r = 0.4) P1 system on [-a,a]^3, n^3 cubes:
//       GMRES (num/krylovsolver.h:320-463) with JACPcCL on M + A + h C_n, right
//       and left preconditioned; the 2x2 Cahn-Hilliard block matrix of
//       surfphasesep/surfphasesep.cpp:431-434 built by the block constructor
//       (num/spmat.h:718-750) and solved by GMRES(50); <steps> warm-started
//       BDF1 steps (surfphasesep.cpp:414-440), plain and with degenerate
//       mobility + wind.  The block solves use a nodal 2x2 block-Jacobi
//       preconditioner written here (DROPS's own driver preconditions with a
//       KLU factorisation through Trilinos, which is not buildable).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <map>
#include <memory>
#include <random>
#include <string>
#include <utility>
#include <valarray>
#include <vector>
#include <unordered_map>
#include <list>
#include <set>
#include <sstream>
#include <tuple>
#include <array>

// The P2 scalar Laplace-Beltrami and C_n forms are not members of
// LocalAssembler; they are built from its own private builders below, which
// is why this file is compiled with -fno-access-control.
#include "geom/builder.h"
#include "misc/problem.h"
#include "levelset/adaptriang.h"
#include "levelset/levelsetmapper.h"
#include "levelset/marking_strategy.h"
#include "num/gradient_recovery.h"
#include "num/krylovsolver.h"
#include "num/precond.h"
#include "surfactant/ifacetransp.h"

using namespace DROPS;

namespace {

struct Writer {
    FILE* f;
    explicit Writer(const char* path) : f(std::fopen(path, "wb")) {
        if (!f) throw std::runtime_error("cannot open output");
        std::fwrite("TFG1", 1, 4, f);
    }
    ~Writer() { std::fclose(f); }
    void put(const std::string& name, char type, const void* data, uint64_t n, size_t es) {
        uint32_t l = (uint32_t)name.size();
        std::fwrite(&l, 4, 1, f);
        std::fwrite(name.data(), 1, l, f);
        std::fwrite(&type, 1, 1, f);
        std::fwrite(&n, 8, 1, f);
        if (n) std::fwrite(data, es, n, f);
    }
    void d(const std::string& name, const std::vector<double>& v) { put(name, 'd', v.data(), v.size(), 8); }
    void l(const std::string& name, const std::vector<int64_t>& v) { put(name, 'l', v.data(), v.size(), 8); }
    void s(const std::string& name, double x) { d(name, std::vector<double>(1, x)); }
    void i(const std::string& name, int64_t x) { l(name, std::vector<int64_t>(1, x)); }
};

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// level sets (surfactant/Surface.hpp:71,130)
// concentration for the degenerate mobility of LaplaceM_P1P1: values in
// about [-0.2, 1.2], so the cut-off at 0 of chi (1 - chi) is exercised
double chi_value(const Point3DCL& x) { return 0.5 + 0.7 * std::sin(2.0 * x[0] + 0.5) * std::cos(1.5 * x[1]) + 0.1 * x[2]; }

// smooth test wind for N_P1P1 (not tangential: the form takes any field)
Point3DCL wind_value(const Point3DCL& x) {
    return Point3DCL(-x[1] + 0.2 * x[2], x[0] - 0.1, 0.3 * x[0] * x[1] + 0.05);
}

double ls_value(const std::string& shape, const Point3DCL& x) {
    if (shape == "sphere") return x.norm() - 1.0;
    if (shape == "torus") {  // R = 1, r = 0.4, symmetry axis z
        double rho = std::sqrt(x[0] * x[0] + x[1] * x[1]) - 1.0;
        return std::sqrt(rho * rho + x[2] * x[2]) - 0.4;
    }
    throw std::invalid_argument("unknown shape");
}

void write_csr(Writer& w, const std::string& name, const MatrixCL& A) {
    std::vector<int64_t> rp(A.num_rows() + 1), ci(A.num_nonzeros());
    std::vector<double> v(A.num_nonzeros());
    for (size_t r = 0; r <= A.num_rows(); ++r) rp[r] = (int64_t)A.raw_row()[r];
    for (size_t k = 0; k < A.num_nonzeros(); ++k) {
        ci[k] = (int64_t)A.raw_col()[k];
        v[k] = A.raw_val()[k];
    }
    w.l(name + ".rowptr", rp);
    w.l(name + ".colind", ci);
    w.d(name + ".vals", v);
}

// Mesh as flat arrays: vertex order of the triangulation; per tet the 4 vertex
// indices and, per local edge, its two vertex indices.
struct Flat {
    std::map<const VertexCL*, int64_t> vid;
    std::vector<int64_t> tet_v, tet_ev;
    std::vector<double> coords;
};
Flat flatten(MultiGridCL& mg, int L = 0) {
    Flat F;
    int64_t k = 0;
    DROPS_FOR_TRIANG_VERTEX(mg, L, it) {
        F.vid[&*it] = k++;
        for (int c = 0; c < 3; ++c) F.coords.push_back(it->GetCoord()[c]);
    }
    DROPS_FOR_TRIANG_TETRA(mg, L, it) {
        for (int i = 0; i < 4; ++i) F.tet_v.push_back(F.vid[it->GetVertex(i)]);
        for (int e = 0; e < 6; ++e) {
            F.tet_ev.push_back(F.vid[it->GetEdge(e)->GetVertex(0)]);
            F.tet_ev.push_back(F.vid[it->GetEdge(e)->GetVertex(1)]);
        }
    }
    return F;
}

// P2 forms built from LocalAssembler's own builders.
LocalAssembler::mtx A_P2P2(LocalAssembler& a) {
    if (a.qDomain.empty()) return a.createMtx(10, 0.);
    a.require(a.qSurfGradP2[0], &LocalAssembler::buildSurfGradP2);
    auto A = a.createMtx(10);
    for (size_t i = 0; i < 10; ++i)
        for (size_t j = i; j < 10; ++j) {
            A[i][j] = quad_2D(dot(a.qSurfGradP2[j], a.qSurfGradP2[i]), a.qDomain);
            A[j][i] = A[i][j];
        }
    return A;
}
LocalAssembler::mtx C_n_P2P2(LocalAssembler& a) {
    a.require(a.q3DGradP2[0], &LocalAssembler::buildGradP2);
    a.require(a.q3DNormal, &LocalAssembler::build3DNormal);
    auto A = a.createMtx(10);
    for (size_t i = 0; i < 10; ++i)
        for (size_t j = i; j < 10; ++j) {
            A[i][j] = quad(dot(a.q3DNormal, a.q3DGradP2[j]) * dot(a.q3DNormal, a.q3DGradP2[i]), a.absDet, a.q3Domain,
                           AllTetraC);
            A[j][i] = A[i][j];
        }
    return A;
}
LocalAssembler::vec F_P2(LocalAssembler& a) {
    if (a.qDomain.empty()) return LocalAssembler::vec(10, 0.);
    a.require(a.qHatP2[0], &LocalAssembler::buildHatP2);
    a.require(a.qConcentrationF, &LocalAssembler::buildConcentrationF);
    LocalAssembler::vec b(10);
    for (size_t i = 0; i < 10; ++i) b[i] = quad_2D(a.qConcentrationF * a.qHatP2[i], a.qDomain);
    return b;
}

int cmd_system(int argc, char** argv) {
    // "system_ref": three more arguments before <out> (width, coarse and fine
    // level): the brick is first refined towards the surface as the
    // surfphasesep driver does (surfphasesep.cpp:170-181: AdapTriangCL with
    // DistMarkingStrategyCL on the distance function, MakeInitialTriang), and
    // everything below runs on the last triangulation level.
    const bool refine = std::string(argv[1]) == "system_ref";
    if (argc < (refine ? 12 : 9))
        throw std::invalid_argument("usage: system p1|p2 lsP1|lsP2 shape n a solve out | "
                                    "system_ref p1|p2 lsP1|lsP2 shape n a solve width coarse fine out");
    const bool p2 = std::string(argv[2]) == "p2";
    const bool lsp2 = std::string(argv[3]) == "lsP2";
    const std::string shape = argv[4];
    const int n = std::atoi(argv[5]);
    const double a = std::atof(argv[6]);
    const int solve_arg = std::atoi(argv[7]);  // -1: the mesh only
    const bool solve = solve_arg > 0;
    Writer w(argv[refine ? 11 : 8]);

    double t0 = now();
    BrickBuilderCL brick(Point3DCL(-a), 2. * a * std_basis<3>(1), 2. * a * std_basis<3>(2), 2. * a * std_basis<3>(3), n, n,
                         n);
    MultiGridCL mg(brick);
    if (refine) {
        const double width = std::atof(argv[8]);
        const int clevel = std::atoi(argv[9]), flevel = std::atoi(argv[10]);
        AdapTriangCL adap(mg);
        DistMarkingStrategyCL marker([&](Point3DCL const& x, double) { return ls_value(shape, x); }, width, clevel,
                                     flevel);
        adap.set_marking_strategy(&marker);
        t0 = now();
        adap.MakeInitialTriang();
        w.s("time_refine", now() - t0);
        adap.set_marking_strategy(nullptr);
        std::vector<int64_t> per_level;
        for (int l = 0; l <= (int)mg.GetLastLevel(); ++l) {
            int64_t c = 0;
            for (auto it = mg.GetTetrasBegin(l), e = mg.GetTetrasEnd(l); it != e; ++it) ++c;
            per_level.push_back(c);
        }
        w.l("tets_per_level", per_level);
        std::vector<int64_t> tl;
        DROPS_FOR_TRIANG_TETRA(mg, (int)mg.GetLastLevel(), it) tl.push_back((int64_t)it->GetLevel());
        w.l("tet_level", tl);
    }
    const int L = (int)mg.GetLastLevel();
    Flat F = flatten(mg, L);
    w.l("tet_v", F.tet_v);
    w.l("tet_ev", F.tet_ev);
    w.d("coords", F.coords);
    w.s("time_mesh", now() - t0);
    if (solve_arg < 0) return 0;

    FESystem sys;
    auto& levelSet = sys.params.levelSet;
    IdxDescCL lsIdx(P2_FE);
    lsIdx.DistributeDOFs(L, mg);
    levelSet.SetIdx(&lsIdx);
    const Uint li = lsIdx.GetIdx();
    // vertex values, then edges: P2 nodal (LSInit) or P1-linear (LinearLSInit),
    // surfactant/surfactant.cpp:733-758.
    DROPS_FOR_TRIANG_VERTEX(mg, L, it) levelSet.Data[it->Unknowns(li)] = ls_value(shape, it->GetCoord());
    DROPS_FOR_TRIANG_EDGE(mg, L, it) {
        if (lsp2)
            levelSet.Data[it->Unknowns(li)] =
                ls_value(shape, 0.5 * (it->GetVertex(0)->GetCoord() + it->GetVertex(1)->GetCoord()));
        else
            levelSet.Data[it->Unknowns(li)] = 0.5 * (levelSet.Data[it->GetVertex(0)->Unknowns(li)] +
                                                     levelSet.Data[it->GetVertex(1)->Unknowns(li)]);
    }
    {
        std::vector<double> lv, le;
        std::vector<int64_t> ev;
        DROPS_FOR_TRIANG_VERTEX(mg, L, it) lv.push_back(levelSet.Data[it->Unknowns(li)]);
        DROPS_FOR_TRIANG_EDGE(mg, L, it) {
            le.push_back(levelSet.Data[it->Unknowns(li)]);
            ev.push_back(F.vid[it->GetVertex(0)]);
            ev.push_back(F.vid[it->GetVertex(1)]);
        }
        w.d("ls_vert", lv);
        w.d("ls_edge", le);
        w.l("edge_v", ev);
    }

    IdxDescCL ifIdx(p2 ? P2IF_FE : P1IF_FE);
    t0 = now();
    size_t n_active = ifIdx.DistributeDOFs(L, mg, &levelSet);
    w.s("time_dofs", now() - t0);
    w.i("n_active", (int64_t)n_active);
    w.i("n_dofs", (int64_t)ifIdx.NumUnknowns());
    {
        std::vector<int64_t> l2g;
        std::vector<int64_t> act;
        int64_t k = 0;
        DROPS_FOR_TRIANG_TETRA(mg, L, it) {
            auto I = ifIdx.Loc2Glo(*it);
            if (!I.empty()) {
                act.push_back(k);
                for (auto x : I) l2g.push_back((int64_t)x);
            }
            ++k;
        }
        w.l("active_tets", act);
        w.l("loc2glo", l2g);
    }

    const double h = 2. * a / n;
    // rhs: f = 13 xyz at ext(x) on the unit sphere (Surface.hpp:46-52)
    sys.params.surfCahnHilliardParams.f = [](Point3DCL const& x, double) {
        Point3DCL y = x - (x.norm() - 1.0) * (x / x.norm());
        return 13. * y[0] * y[1] * y[2];
    };
    MatrixCL Mm, Am, Cm, Nm;
    VectorCL rhs;
    double t_asm = 0.;
    t0 = now();
    if (!p2) {
        FEMatDescCL M(&ifIdx, &ifIdx, &LocalAssembler::M_P1P1), A(&ifIdx, &ifIdx, &LocalAssembler::A_P1P1),
            C(&ifIdx, &ifIdx, &LocalAssembler::C_n_P1P1);
        FEVecDescCL f(&ifIdx, &LocalAssembler::F_concentration_P1);
        sys.matrices = {&M, &A, &C};
        sys.vectors = {&f};
        setupFESystem(mg, sys);
        Mm = M.Data;
        Am = A.Data;
        Cm = C.Data;
        rhs.resize(f.Data.size());
        rhs = f.Data;
        t_asm = now() - t0;
        // wind convection N_P1P1 (surfactant/ifacetransp.h:1590-1600) with a
        // vecP2IF wind interpolated as in surfphasesep/surfphasesep.cpp:198-213, 417-420
        IdxDescCL velIdx(vecP2IF_FE);
        velIdx.DistributeDOFs(L, mg, &levelSet);
        VecDescCL wind(&velIdx);
        wind.Interpolate(mg, [](Point3DCL const& x) { return wind_value(x); });
        FESystem nsys;
        nsys.params.levelSet.SetIdx(&lsIdx);
        nsys.params.levelSet.Data = levelSet.Data;
        nsys.params.surfCahnHilliardParams.u_T = &wind;
        FEMatDescCL N(&ifIdx, &ifIdx, &LocalAssembler::N_P1P1);
        nsys.matrices = {&N};
        setupFESystem(mg, nsys);
        Nm = N.Data;
        write_csr(w, "N", Nm);
        // LaplaceM_P1P1 (:1533-1544) with the degenerate mobility chi (1 - chi),
        // cut off at 0 (buildMobility :1176-1190), chi interpolated on the
        // interface index
        {
            VecDescCL chi(&ifIdx);
            chi.Interpolate(mg, [](Point3DCL const& x) { return chi_value(x); });
            FESystem lsys;
            lsys.params.levelSet.SetIdx(&lsIdx);
            lsys.params.levelSet.Data = levelSet.Data;
            lsys.params.surfCahnHilliardParams.useDegenerateMobility = true;
            lsys.params.surfCahnHilliardParams.chi = &chi;
            FEMatDescCL L(&ifIdx, &ifIdx, &LocalAssembler::LaplaceM_P1P1);
            lsys.matrices = {&L};
            setupFESystem(mg, lsys);
            write_csr(w, "LapM", L.Data);
            w.d("chi", std::vector<double>(std::begin(chi.Data), std::end(chi.Data)));
        }
        std::vector<double> wv, we;
        DROPS_FOR_TRIANG_VERTEX(mg, L, it) {
            const Point3DCL v = wind_value(it->GetCoord());
            for (int c = 0; c < 3; ++c) wv.push_back(v[c]);
        }
        DROPS_FOR_TRIANG_EDGE(mg, L, it) {
            const Point3DCL v = wind_value(GetBaryCenter(*it));
            for (int c = 0; c < 3; ++c) we.push_back(v[c]);
        }
        w.d("wind_vert", wv);
        w.d("wind_edge", we);
    } else {
        // FESystemAccumulator::visit restated for the P2 forms above
        const size_t m = ifIdx.NumUnknowns();
        MatrixBuilderCL bM(&Mm, m, m), bA(&Am, m, m), bC(&Cm, m, m);
        rhs.resize(m, 0.);
        DROPS_FOR_TRIANG_TETRA(mg, L, it) {
            auto I = ifIdx.Loc2Glo(*it);
            if (I.empty()) continue;
            LocalAssembler as(*it, sys.params);
            auto fm = as.M_P2P2();
            auto fa = A_P2P2(as);
            auto fc = C_n_P2P2(as);
            auto fb = F_P2(as);
            for (size_t i = 0; i < 10; ++i) {
                for (size_t j = 0; j < 10; ++j) {
                    bM(I[i], I[j]) += fm[i][j];
                    bA(I[i], I[j]) += fa[i][j];
                    bC(I[i], I[j]) += fc[i][j];
                }
                rhs[I[i]] += fb[i];
            }
        }
        bM.Build();
        bA.Build();
        bC.Build();
    }
    if (p2) t_asm = now() - t0;
    w.s("time_assemble", t_asm);
    write_csr(w, "M", Mm);
    write_csr(w, "A", Am);
    write_csr(w, "C", Cm);
    w.d("rhs", std::vector<double>(std::begin(rhs), std::end(rhs)));

    if (solve) {
        MatrixCL S(1., Mm, 1., Am, h, Cm);  // LinComb ctor (num/spmat.h:712-715)
        write_csr(w, "S", S);
        VectorCL x(0., S.num_rows());
        JACPcCL pc;
        PCGSolverCL<JACPcCL> solver(pc, 100000, 1e-10, true);
        t0 = now();
        solver.Solve(S, x, rhs, ifIdx.GetEx());
        w.s("time_solve", now() - t0);
        w.i("iters", solver.GetIter());
        w.s("resid", solver.GetResid());
        w.d("x", std::vector<double>(std::begin(x), std::end(x)));
        // the solution as VecDescCL::Write writes it, binary (misc/problem.h:928-944)
        VecDescCL xv(&ifIdx);
        xv.Data = x;
        std::ofstream vf(std::string(argv[argc - 1]) + ".vec", std::ios::binary);
        xv.Write(vf, true);
    }
    return 0;
}

double plane(const Point3DCL& p) { return p[0] - 0.41; }
double plane2(const Point3DCL& p) { return p[0] - 0.4; }
double sphere_2(const Point3DCL& p) { return (p - Point3DCL(0.5)).norm() - 0.31; }

// tests/interfaceP1FE.cpp restated without LevelsetP2CL: P2 level set by
// nodal interpolation, numbering by IdxDescCL::CreateNumbering (P1IF_FE).
int cmd_legacy_numb(int argc, char** argv) {
    if (argc < 4) throw std::invalid_argument("usage: legacy_numb case out");
    const std::string cs = argv[2];
    Writer w(argv[3]);
    int nx = 10, ny = 1, nz = 1;
    std::function<double(const Point3DCL&)> fn = plane;
    if (cs == "plane2") fn = plane2;
    if (cs == "sphere") { nx = ny = nz = 20; fn = sphere_2; }
    BrickBuilderCL brick(std_basis<3>(0), std_basis<3>(1), std_basis<3>(2), std_basis<3>(3), nx, ny, nz);
    MultiGridCL mg(brick);
    Flat F = flatten(mg);
    w.l("tet_v", F.tet_v);
    w.l("tet_ev", F.tet_ev);
    w.d("coords", F.coords);
    IdxDescCL lsIdx(P2_FE);
    lsIdx.DistributeDOFs(0, mg);
    VecDescCL ls(&lsIdx);
    const Uint li = lsIdx.GetIdx();
    DROPS_FOR_TRIANG_VERTEX(mg, 0, it) ls.Data[it->Unknowns(li)] = fn(it->GetCoord());
    DROPS_FOR_TRIANG_EDGE(mg, 0, it)
        ls.Data[it->Unknowns(li)] = fn(0.5 * (it->GetVertex(0)->GetCoord() + it->GetVertex(1)->GetCoord()));
    BndCondT bc[6] = {NoBC, NoBC, NoBC, NoBC, NoBC, NoBC};
    BndDataCL<> lsbnd(6, bc);
    IdxDescCL ifIdx(P1IF_FE);
    int64_t status = 0, n_active = -1, n_dofs = -1;
    try {
        n_active = (int64_t)ifIdx.CreateNumbering(0, mg, &ls, &lsbnd);
        n_dofs = (int64_t)ifIdx.NumUnknowns();
    } catch (std::exception& e) {
        status = 2;
        std::cerr << "legacy_numb: " << e.what() << "\n";
    } catch (DROPSErrCL& e) {
        status = 3;
    }
    w.i("status", status);
    w.i("n_active", n_active);
    w.i("n_dofs", n_dofs);
    if (status == 0) {
        std::vector<int64_t> dv;
        const Uint ii = ifIdx.GetIdx();
        DROPS_FOR_TRIANG_VERTEX(mg, 0, it) dv.push_back(it->Unknowns.Exist(ii) ? (int64_t)it->Unknowns(ii) : -1);
        w.l("dof_vert", dv);
    }
    return 0;
}

double legacy_f(const Point3DCL& p, double) { return 1.0 + p[0] * p[1] - 0.5 * p[2]; }

// The older surfactant.cpp path: legacy numbering and the legacy P1 forms.
int cmd_legacy_forms(int argc, char** argv) {
    if (argc < 5) throw std::invalid_argument("usage: legacy_forms n a out");
    const int n = std::atoi(argv[2]);
    const double a = std::atof(argv[3]);
    Writer w(argv[4]);
    BrickBuilderCL brick(Point3DCL(-a), 2. * a * std_basis<3>(1), 2. * a * std_basis<3>(2), 2. * a * std_basis<3>(3), n,
                         n, n);
    MultiGridCL mg(brick);
    Flat F = flatten(mg);
    w.l("tet_v", F.tet_v);
    w.l("tet_ev", F.tet_ev);
    w.d("coords", F.coords);
    IdxDescCL lsIdx(P2_FE);
    lsIdx.DistributeDOFs(0, mg);
    VecDescCL ls(&lsIdx);
    const Uint li = lsIdx.GetIdx();
    DROPS_FOR_TRIANG_VERTEX(mg, 0, it) ls.Data[it->Unknowns(li)] = it->GetCoord().norm() - 1.0;
    DROPS_FOR_TRIANG_EDGE(mg, 0, it)
        ls.Data[it->Unknowns(li)] = (0.5 * (it->GetVertex(0)->GetCoord() + it->GetVertex(1)->GetCoord())).norm() - 1.0;
    BndCondT bc[6] = {NoBC, NoBC, NoBC, NoBC, NoBC, NoBC};
    BndDataCL<> lsbnd(6, bc);
    IdxDescCL ifIdx(P1IF_FE);
    const int64_t n_active = (int64_t)ifIdx.CreateNumbering(0, mg, &ls, &lsbnd);
    w.i("n_active", n_active);
    w.i("n_dofs", (int64_t)ifIdx.NumUnknowns());
    std::vector<int64_t> dv;
    const Uint ii = ifIdx.GetIdx();
    DROPS_FOR_TRIANG_VERTEX(mg, 0, it) dv.push_back(it->Unknowns.Exist(ii) ? (int64_t)it->Unknowns(ii) : -1);
    w.l("dof_vert", dv);
    std::vector<double> lsv, lse;
    DROPS_FOR_TRIANG_VERTEX(mg, 0, it) lsv.push_back(ls.Data[it->Unknowns(li)]);
    w.d("ls_vert", lsv);
    std::vector<int64_t> ev;
    DROPS_FOR_TRIANG_EDGE(mg, 0, it) {
        lse.push_back(ls.Data[it->Unknowns(li)]);
        ev.push_back(F.vid[it->GetVertex(0)]);
        ev.push_back(F.vid[it->GetVertex(1)]);
    }
    w.d("ls_edge", lse);
    w.l("edge_v", ev);
    const double alpha = 0.7, D = 1.3;
    w.s("alpha", alpha);
    w.s("D", D);
    MatDescCL M(&ifIdx, &ifIdx), A(&ifIdx, &ifIdx);
    SetupInterfaceMassP1(mg, &M, ls, lsbnd, alpha);
    SetupLBP1(mg, &A, ls, lsbnd, D);
    write_csr(w, "M", M.Data);
    write_csr(w, "A", A.Data);
    VecDescCL rhs(&ifIdx);
    SetupInterfaceRhsP1(mg, &rhs, ls, lsbnd, legacy_f, 0.);
    w.d("rhs", std::vector<double>(std::begin(rhs.Data), std::end(rhs.Data)));
    return 0;
}

// tests/principallattice.cpp:316-347 (sphere r = 0.5 on [-1,1]^3, 8^3 cubes)
int cmd_area(int argc, char** argv) {
    if (argc < 3) throw std::invalid_argument("usage: area out");
    Writer w(argv[2]);
    BrickBuilderCL brick(Point3DCL(-1.), 2. * std_basis<3>(1), 2. * std_basis<3>(2), 2. * std_basis<3>(3), 8, 8, 8);
    MultiGridCL mg(brick);
    const PrincipalLatticeCL& lat = PrincipalLatticeCL::instance(2);
    GridFunctionCL<> ls(lat.vertex_size());
    SurfacePatchCL patch;
    QuadDomain2DCL qdom;
    double surf = 0.;
    std::vector<double> per_tet;
    std::vector<int64_t> nfac;
    auto sph = [](const Point3DCL& p, double) { return p.norm() - 0.5; };
    DROPS_FOR_TRIANG_TETRA(mg, 0, it) {
        evaluate_on_vertexes(InstatScalarFunction(sph), *it, lat, 0., Addr(ls));
        patch.make_patch<MergeCutPolicyCL>(lat, ls);
        make_CompositeQuad5Domain2D(qdom, patch, *it);
        GridFunctionCL<> integrand(1., qdom.vertex_size());
        double s = quad_2D(integrand, qdom);
        surf += s;
        per_tet.push_back(s);
        nfac.push_back(patch.facet_size());
    }
    w.s("surface", surf);
    w.d("per_tet", per_tet);
    w.l("n_facets", nfac);
    Flat F = flatten(mg);
    w.l("tet_v", F.tet_v);
    w.l("tet_ev", F.tet_ev);
    w.d("coords", F.coords);
    // the patch topology of the first cut tets, for the patch parity test
    std::vector<int64_t> facets, bnd, tet_of;
    std::vector<double> verts;
    std::vector<int64_t> nverts;
    int64_t k = 0, dumped = 0;
    DROPS_FOR_TRIANG_TETRA(mg, 0, it) {
        evaluate_on_vertexes(InstatScalarFunction(sph), *it, lat, 0., Addr(ls));
        patch.make_patch<MergeCutPolicyCL>(lat, ls);
        if (!patch.empty() && dumped < 400) {
            tet_of.push_back(k);
            nverts.push_back(patch.vertex_size());
            for (auto f = patch.facet_begin(); f != patch.facet_end(); ++f) {
                for (int j = 0; j < 3; ++j) facets.push_back((*f)[j]);
                bnd.push_back(patch.is_boundary_facet(f) ? 1 : 0);
            }
            for (auto v = patch.vertex_begin(); v != patch.vertex_end(); ++v)
                for (int c = 0; c < 4; ++c) verts.push_back((*v)[c]);
            std::vector<double> lsv(std::begin(ls), std::end(ls));
            ++dumped;
        }
        ++k;
    }
    w.l("patch_tets", tet_of);
    w.l("patch_nverts", nverts);
    w.l("patch_facets", facets);
    w.l("patch_boundary", bnd);
    w.d("patch_verts", verts);
    return 0;
}

// Nodal 2x2 block Jacobi for a 2x2 block system of size 2h: for DOF i the
// inverse of [[B(i,i), B(i,i+h)], [B(i+h,i), B(i+h,i+h)]] applied to
// (b_i, b_{i+h}).  Test infrastructure with the Apply(A, x, b, ex) interface
// that DROPS's GMRES calls on its preconditioner.
class NodalBlockJacobiPcCL {
    std::vector<double> inv_;
    size_t h_ = 0;

  public:
    explicit NodalBlockJacobiPcCL(const MatrixCL& B) : inv_(2 * B.num_rows()), h_(B.num_rows() / 2) {
        auto at = [&](size_t r, size_t c) {
            for (size_t k = B.raw_row()[r]; k < B.raw_row()[r + 1]; ++k)
                if (B.raw_col()[k] == c) return B.raw_val()[k];
            return 0.;
        };
        for (size_t i = 0; i < h_; ++i) {
            const double a11 = at(i, i), a12 = at(i, i + h_), a21 = at(i + h_, i), a22 = at(i + h_, i + h_);
            const double det = a11 * a22 - a12 * a21;
            inv_[4 * i] = a22 / det;
            inv_[4 * i + 1] = -a12 / det;
            inv_[4 * i + 2] = -a21 / det;
            inv_[4 * i + 3] = a11 / det;
        }
    }
    template <typename Mat, typename Vec, typename ExT>
    void Apply(const Mat&, Vec& x, const Vec& b, const ExT&) const {
        for (size_t i = 0; i < h_; ++i) {
            const double u = b[i], v = b[i + h_];
            x[i] = inv_[4 * i] * u + inv_[4 * i + 1] * v;
            x[i + h_] = inv_[4 * i + 2] * u + inv_[4 * i + 3] * v;
        }
    }
};

int cmd_gmres(int argc, char** argv) {
    // "gmres_ref": the brick first refined towards the torus (width, coarse
    // and fine level before <out>, surfphasesep.cpp:170-181), everything on
    // the last level
    const bool refine = std::string(argv[1]) == "gmres_ref";
    if (argc < (refine ? 9 : 6))
        throw std::invalid_argument("usage: gmres n a steps out | gmres_ref n a steps width coarse fine out");
    const int n = std::atoi(argv[2]);
    const double a = std::atof(argv[3]);
    const int steps = std::atoi(argv[4]);
    Writer w(argv[refine ? 8 : 5]);

    BrickBuilderCL brick(Point3DCL(-a), 2. * a * std_basis<3>(1), 2. * a * std_basis<3>(2), 2. * a * std_basis<3>(3), n, n,
                         n);
    MultiGridCL mg(brick);
    if (refine) {
        AdapTriangCL adap(mg);
        DistMarkingStrategyCL marker([&](Point3DCL const& x, double) { return ls_value("torus", x); },
                                     std::atof(argv[5]), std::atoi(argv[6]), std::atoi(argv[7]));
        adap.set_marking_strategy(&marker);
        adap.MakeInitialTriang();
        adap.set_marking_strategy(nullptr);
        Flat F = flatten(mg, (int)mg.GetLastLevel());
        w.l("tet_v", F.tet_v);
        w.d("coords", F.coords);
    }
    const int L = (int)mg.GetLastLevel();
    FESystem sys;
    auto& levelSet = sys.params.levelSet;
    IdxDescCL lsIdx(P2_FE);
    lsIdx.DistributeDOFs(L, mg);
    levelSet.SetIdx(&lsIdx);
    const Uint li = lsIdx.GetIdx();
    // P1 level set stored as a P2 vector (LinearLSInit, surfactant/surfactant.cpp:748-758)
    DROPS_FOR_TRIANG_VERTEX(mg, L, it) levelSet.Data[it->Unknowns(li)] = ls_value("torus", it->GetCoord());
    DROPS_FOR_TRIANG_EDGE(mg, L, it)
        levelSet.Data[it->Unknowns(li)] = 0.5 * (levelSet.Data[it->GetVertex(0)->Unknowns(li)] +
                                                 levelSet.Data[it->GetVertex(1)->Unknowns(li)]);
    IdxDescCL ifIdx(P1IF_FE);
    ifIdx.DistributeDOFs(L, mg, &levelSet);
    const size_t m = ifIdx.NumUnknowns();
    w.i("n_dofs", (int64_t)m);
    sys.params.surfCahnHilliardParams.f = [](Point3DCL const& x, double) {
        Point3DCL y = x - (x.norm() - 1.0) * (x / x.norm());
        return 13. * y[0] * y[1] * y[2];
    };
    FEMatDescCL M(&ifIdx, &ifIdx, &LocalAssembler::M_P1P1), A(&ifIdx, &ifIdx, &LocalAssembler::A_P1P1),
        C(&ifIdx, &ifIdx, &LocalAssembler::C_n_P1P1);
    FEVecDescCL f(&ifIdx, &LocalAssembler::F_concentration_P1);
    sys.matrices = {&M, &A, &C};
    sys.vectors = {&f};
    setupFESystem(mg, sys);
    write_csr(w, "M", M.Data);
    const double h = 2. * a / n;

    // GMRES(20) with point Jacobi on the surface Poisson system, both preconditioning sides
    {
        MatrixCL S(1., M.Data, 1., A.Data, h, C.Data);
        write_csr(w, "S", S);
        w.d("rhs", std::vector<double>(std::begin(f.Data), std::end(f.Data)));
        JACPcCL pc;
        const char* side[2] = {"right", "left"};
        for (int s = 0; s < 2; ++s) {
            VectorCL x(0., m);
            int it = 100000;
            double tol = 1e-10;
            const bool ok = GMRES(S, x, f.Data, ifIdx.GetEx(), pc, 20, it, tol, true, false,
                                  s == 0 ? RightPreconditioning : LeftPreconditioning);
            w.i(std::string("gmres_") + side[s] + "_ok", ok ? 1 : 0);
            w.i(std::string("gmres_") + side[s] + "_iters", it);
            w.s(std::string("gmres_") + side[s] + "_resid", tol);
            w.d(std::string("gmres_") + side[s] + "_x", std::vector<double>(std::begin(x), std::end(x)));
        }
    }

    // Cahn-Hilliard: dt = 1e-3, mobility 1, eps = 0.02, rho_vol = h, beta_s = 0, xi = 1
    const double dt = 1e-3, alpha = 1. / dt, mob = 1., eps = 0.02, rho = h, beta_s = 0., xi = 1.;
    w.s("dt", dt);
    w.s("eps", eps);
    w.s("rho", rho);
    w.s("beta_s", beta_s);
    w.s("xi", xi);
    auto chemicalPotential = [&](double c) { return xi * 2 * c * (1 - c) * (1 - 2 * c); };  // surfphasesep.cpp:140-151
    auto block = [&](const MatrixCL& UL, const MatrixCL& Amob) {  // surfphasesep.cpp:431-434
        return MatrixCL(UL, MatrixCL(mob, Amob, rho, C.Data), MatrixCL(eps * eps, A.Data, beta_s, M.Data, eps * eps * rho, C.Data),
                        MatrixCL(-1., M.Data));
    };
    // right-hand side of a BDF1 step from chi (surfphasesep.cpp:421-425, f = 0)
    auto rhs_of = [&](const VectorCL& chi) {
        VectorCL F_chi((1. / dt) * (M.Data * chi));
        VectorCL fp(m);
        for (size_t i = 0; i < m; ++i) fp[i] = chemicalPotential(chi[i]);
        VectorCL F_omega(beta_s * (M.Data * chi) - M.Data * fp);
        VectorCL b(2 * m);
        b[std::slice(0, m, 1)] = F_chi;
        b[std::slice(m, m, 1)] = F_omega;
        return b;
    };
    auto solve = [&](const MatrixCL& B, VectorCL& x, const VectorCL& b, int& it, double& tol) {
        NodalBlockJacobiPcCL pc(B);
        it = 20000;
        tol = 1e-10;
        return GMRES(B, x, b, ifIdx.GetEx(), pc, 50, it, tol, true, false, RightPreconditioning);
    };
    std::mt19937_64 rng(11);
    std::uniform_real_distribution<double> U(-0.01, 0.01);
    VectorCL chi0(m);
    for (size_t i = 0; i < m; ++i) chi0[i] = 0.5 + U(rng);
    w.d("chi0", std::vector<double>(std::begin(chi0), std::end(chi0)));
    {
        const MatrixCL B = block(MatrixCL(alpha, M.Data), A.Data);
        write_csr(w, "B", B);
        // one solve from a zero initial guess
        VectorCL x(0., 2 * m);
        int it;
        double tol;
        const bool ok = solve(B, x, rhs_of(chi0), it, tol);
        w.i("block_ok", ok ? 1 : 0);
        w.i("block_iters", it);
        w.s("block_resid", tol);
        w.d("block_x", std::vector<double>(std::begin(x), std::end(x)));
        // BDF1 steps, each warm-started from the previous [chi; omega]
        VectorCL X(0., 2 * m);
        X[std::slice(0, m, 1)] = chi0;
        std::vector<int64_t> its;
        std::vector<double> res, states;
        for (int k = 0; k < steps; ++k) {
            VectorCL chi(X[std::slice(0, m, 1)]);
            if (!solve(B, X, rhs_of(chi), it, tol)) throw std::runtime_error("BDF1 step did not converge");
            its.push_back(it);
            res.push_back(tol);
            states.insert(states.end(), std::begin(X), std::end(X));
        }
        w.l("steps_iters", its);
        w.d("steps_resid", res);
        w.d("steps_X", states);
    }
    // BDF1 steps with degenerate mobility (LaplaceM_P1P1 from the current chi,
    // surfactant/ifacetransp.h:1533-1544) and wind convection N_P1P1 (:1590-1600)
    {
        IdxDescCL velIdx(vecP2IF_FE);
        velIdx.DistributeDOFs(L, mg, &levelSet);
        VecDescCL wind(&velIdx);
        wind.Interpolate(mg, [](Point3DCL const& x) { return wind_value(x); });
        std::uniform_real_distribution<double> U3(-0.3, 0.3);
        std::mt19937_64 rng3(9);
        VectorCL X(0., 2 * m);
        for (size_t i = 0; i < m; ++i) X[i] = 0.5 + U3(rng3);
        w.d("dm_chi0", std::vector<double>(std::begin(X), std::begin(X) + m));
        VecDescCL chi(&ifIdx);
        std::vector<int64_t> its;
        std::vector<double> res, states;
        for (int k = 0; k < steps; ++k) {
            chi.Data = VectorCL(X[std::slice(0, m, 1)]);
            FESystem csys;
            csys.params.levelSet.SetIdx(&lsIdx);
            csys.params.levelSet.Data = levelSet.Data;
            csys.params.surfCahnHilliardParams.useDegenerateMobility = true;
            csys.params.surfCahnHilliardParams.chi = &chi;
            csys.params.surfCahnHilliardParams.u_T = &wind;
            FEMatDescCL Adeg(&ifIdx, &ifIdx, &LocalAssembler::LaplaceM_P1P1), N(&ifIdx, &ifIdx, &LocalAssembler::N_P1P1);
            csys.matrices = {&Adeg, &N};
            setupFESystem(mg, csys);
            const MatrixCL B = block(MatrixCL(alpha, M.Data, 1., N.Data), Adeg.Data);
            if (k == 0) write_csr(w, "dm_B0", B);
            int it;
            double tol;
            if (!solve(B, X, rhs_of(chi.Data), it, tol)) throw std::runtime_error("BDF1 step did not converge");
            its.push_back(it);
            res.push_back(tol);
            states.insert(states.end(), std::begin(X), std::end(X));
        }
        w.l("dm_steps_iters", its);
        w.d("dm_steps_resid", res);
        w.d("dm_steps_X", states);
    }
    return 0;
}

// f = 13 xyz on the unit sphere at the projected points (Surface.hpp:46-52 restated as in cmd_system)
double quaqua_f(const Point3DCL& x, double) { return 13. * x[0] * x[1] * x[2]; }

int cmd_quaqua(int argc, char** argv) {
    if (argc < 5) throw std::invalid_argument("usage: quaqua n a out");
    const int n = std::atoi(argv[2]);
    const double a = std::atof(argv[3]);
    Writer w(argv[4]);
    BrickBuilderCL brick(Point3DCL(-a), 2. * a * std_basis<3>(1), 2. * a * std_basis<3>(2), 2. * a * std_basis<3>(3), n,
                         n, n);
    MultiGridCL mg(brick);
    Flat F = flatten(mg);
    IdxDescCL lsIdx(P2_FE);
    lsIdx.DistributeDOFs(0, mg);
    VecDescCL ls(&lsIdx);
    const Uint li = lsIdx.GetIdx();
    DROPS_FOR_TRIANG_VERTEX(mg, 0, it) ls.Data[it->Unknowns(li)] = ls_value("sphere", it->GetCoord());
    DROPS_FOR_TRIANG_EDGE(mg, 0, it)
        ls.Data[it->Unknowns(li)] = ls_value("sphere", 0.5 * (it->GetVertex(0)->GetCoord() + it->GetVertex(1)->GetCoord()));
    BndCondT bc[6] = {NoBC, NoBC, NoBC, NoBC, NoBC, NoBC};
    BndDataCL<> lsbnd(6, bc);
    {
        std::vector<double> lv, le;
        std::vector<int64_t> ev;
        DROPS_FOR_TRIANG_VERTEX(mg, 0, it) lv.push_back(ls.Data[it->Unknowns(li)]);
        DROPS_FOR_TRIANG_EDGE(mg, 0, it) {
            le.push_back(ls.Data[it->Unknowns(li)]);
            ev.push_back(F.vid[it->GetVertex(0)]);
            ev.push_back(F.vid[it->GetVertex(1)]);
        }
        w.d("ls_vert", lv);
        w.d("ls_edge", le);
        w.l("edge_v", ev);
    }
    // interface P2 numbering (DistributeDOFs, the UH API)
    IdxDescCL ifIdx(P2IF_FE);
    ifIdx.DistributeDOFs(0, mg, &ls);
    w.i("n_dofs", (int64_t)ifIdx.NumUnknowns());
    // recovered gradient of the level set: P2 vector field, nodal averages over the tets
    IdxDescCL vecIdx(vecP2_FE);
    vecIdx.CreateNumbering(0, mg);
    VecDescCL grad(&vecIdx);
    averaging_P2_gradient_recovery(mg, ls, lsbnd, grad);
    {
        const Uint gi = vecIdx.GetIdx();
        std::vector<double> gv, ge;
        DROPS_FOR_TRIANG_VERTEX(mg, 0, it)
            for (int c = 0; c < 3; ++c) gv.push_back(grad.Data[it->Unknowns(gi) + c]);
        DROPS_FOR_TRIANG_EDGE(mg, 0, it)
            for (int c = 0; c < 3; ++c) ge.push_back(grad.Data[it->Unknowns(gi) + c]);
        w.d("grad_vert", gv);
        w.d("grad_edge", ge);
    }
    const PrincipalLatticeCL& lat = PrincipalLatticeCL::instance(1);
    TetraToTetrasT nbh;
    compute_tetra_neighborhoods(mg, ls, lsbnd, lat, nbh);
    // Newton form of the mapper, tolerance far below the one of the reference's parameter files so
    // that every base point is the root to rounding
    QuaQuaMapperCL quaqua(mg, ls, grad, &nbh, 100, 1e-13, false, 1e-4);
    TetraAccumulatorTupleCL accus;
    InterfaceCommonDataP2CL cdata(ls, lsbnd, quaqua, lat);
    accus.push_back(&cdata);
    MatDescCL M(&ifIdx, &ifIdx), A(&ifIdx, &ifIdx);
    InterfaceMatrixAccuCL<LocalMassP2CL, InterfaceCommonDataP2CL> accuM(&M, LocalMassP2CL(), cdata, "Mp2");
    accus.push_back(&accuM);
    InterfaceMatrixAccuCL<LocalLaplaceBeltramiP2CL, InterfaceCommonDataP2CL> accuA(&A, LocalLaplaceBeltramiP2CL(1.0),
                                                                                 cdata, "Ap2");
    accus.push_back(&accuA);
    VecDescCL b(&ifIdx);
    InterfaceVectorAccuCL<LocalVectorP2CL, InterfaceCommonDataP2CL> accub(&b, LocalVectorP2CL(quaqua_f, 0.), cdata);
    accus.push_back(&accub);
    accumulate(accus, mg, ifIdx.TriangLevel(), ifIdx.GetBndInfo());
    write_csr(w, "M", M.Data);
    write_csr(w, "A", A.Data);
    w.d("rhs", std::vector<double>(std::begin(b.Data), std::end(b.Data)));
    return 0;
}

// The 64 refinement rules (geom/topo.h:196-223): per edge pattern the
// children's local points (ChildDataCL::Vertices) in rule order.
int cmd_rules(int argc, char** argv) {
    if (argc < 3) throw std::invalid_argument("usage: rules out");
    Writer w(argv[2]);
    std::vector<int64_t> nch, ch;
    for (Uint p = 0; p < 64; ++p) {
        const RefRuleCL& R = GetRefRule((Ubyte)p);
        nch.push_back(R.ChildNum);
        for (Uint c = 0; c < 8; ++c)
            for (Uint k = 0; k < 4; ++k)
                ch.push_back(c < R.ChildNum ? (int64_t)GetChildData(R.Children[c]).Vertices[k] : -1);
    }
    w.l("nch", nch);
    w.l("children", ch);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    try {
        if (argc < 2) throw std::invalid_argument("usage: ref_harness <cmd> ...");
        std::string cmd = argv[1];
        if (cmd == "system" || cmd == "system_ref") return cmd_system(argc, argv);
        if (cmd == "rules") return cmd_rules(argc, argv);
        if (cmd == "legacy_numb") return cmd_legacy_numb(argc, argv);
        if (cmd == "legacy_forms") return cmd_legacy_forms(argc, argv);
        if (cmd == "area") return cmd_area(argc, argv);
        if (cmd == "gmres" || cmd == "gmres_ref") return cmd_gmres(argc, argv);
        if (cmd == "quaqua") return cmd_quaqua(argc, argv);
        throw std::invalid_argument("unknown command " + cmd);
    } catch (std::exception& e) {
        std::cerr << "ref_harness: " << e.what() << "\n";
        return 1;
    } catch (DROPSErrCL& e) {
        e.handle();
        return 1;
    }
}
