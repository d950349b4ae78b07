// Drop-in GPU versions of the DROPS TraceFEM calls over libtracefem's C ABI
// (declarations and contract in tracefem_drops.h).
#include "tracefem_drops.h"

#include <cstring>
#include <stdexcept>
#include <unordered_map>

namespace DROPS {
namespace gpu {

static_assert(sizeof(size_t) == sizeof(int64_t), "MatrixCL's size_t CSR is passed as int64");

namespace {

struct Session {
    tf_context* ctx = nullptr;
    // what is on the device: the flattened level and its level set
    const MultiGridCL* mg = nullptr;
    Uint level = 0;
    size_t nv = 0, ne = 0, nt = 0;
    const void* ls_data = nullptr;
    size_t ls_size = 0;
    std::vector<double> ls_copy;  // compared element-wise: the caller may change values in place
    // the numbering last computed by DistributeDOFs (index and distance)
    Uint idx_id = static_cast<Uint>(-1);
    double idx_dist = 0.;
    int rhs_kind = TF_RHS_NONE;
    std::vector<double> rhs_par;
    ~Session() {
        if (ctx) tf_destroy(ctx);
    }
};

Session& session() {
    static thread_local Session s;
    return s;
}

void check(int st) {
    if (st == TF_OK) return;
    const std::string msg = std::string("libtracefem: ") + tf_status_string(st) + ": " +
                            (session().ctx ? tf_last_error(session().ctx) : "");
    if (st == TF_ERR_ZERO_NODE) throw std::invalid_argument(msg);  // distance() throws std::invalid_argument
    throw DROPSErrCL(msg);
}

template <class F>
void for_vertices(const MultiGridCL& mg, Uint level, F f) {
    for (auto it = mg.GetTriangVertexBegin(level); it != mg.GetTriangVertexEnd(level); ++it) f(*it);
}
template <class F>
void for_edges(const MultiGridCL& mg, Uint level, F f) {
    for (auto it = mg.GetTriangEdgeBegin(level); it != mg.GetTriangEdgeEnd(level); ++it) f(*it);
}
template <class F>
void for_tets(const MultiGridCL& mg, Uint level, F f) {
    for (auto it = mg.GetTriangTetraBegin(level); it != mg.GetTriangTetraEnd(level); ++it) f(*it);
}

// mesh and P2 level set on the device (uploaded again only when they changed)
void ensure_uploaded(const MultiGridCL& mg, Uint level, const VecDescCL& ls) {
    Session& s = session();
    tf_context* c = context();
    size_t nv = 0, ne = 0, nt = 0;
    for_vertices(mg, level, [&](const VertexCL&) { ++nv; });
    for_edges(mg, level, [&](const EdgeCL&) { ++ne; });
    for_tets(mg, level, [&](const TetraCL&) { ++nt; });
    if (s.mg != &mg || s.level != level || s.nv != nv || s.ne != ne || s.nt != nt) {
        const FlatLevel F = Flatten(mg, level);
        check(tf_mesh_upload(c, (int64_t)nv, F.coords.data(), (int64_t)nt, F.tet_v.data(), F.tet_e.data(),
                             (int64_t)ne, F.edge_v.data()));
        s.mg = &mg;
        s.level = level;
        s.nv = nv;
        s.ne = ne;
        s.nt = nt;
        s.ls_data = nullptr;
    }
    if (s.ls_data != &ls || s.ls_size != ls.Data.size() ||
        (ls.Data.size() && std::memcmp(s.ls_copy.data(), Addr(ls.Data), sizeof(double) * ls.Data.size()))) {
        std::vector<double> lv, le;
        LevelSetValues(mg, level, ls, lv, le);
        check(tf_levelset_upload(c, lv.data(), le.data()));
        s.ls_data = &ls;
        s.ls_size = ls.Data.size();
        s.ls_copy.assign(Addr(ls.Data), Addr(ls.Data) + ls.Data.size());
    }
}

int fe_of(const IdxDescCL& idx) { return idx.NumUnknownsEdge() ? TF_P2IF : TF_P1IF; }

// per-DOF values of a P1IF vector as this library's numbering sees them (identical numbering)
void upload_vec(int vec, const VectorCL& v) {
    check(tf_vec_upload(context(), vec, (int64_t)v.size(), v.size() ? Addr(v) : nullptr));
}

// vecP2IF wind (u_T) at the flattened vertices and edges, xyz; 0 where it has no DOF
void upload_wind(const MultiGridCL& mg, Uint level, const VecDescCL& w) {
    const Uint id = w.RowIdx->GetIdx();
    const size_t block = w.RowIdx->NumUnknowns() / 3;
    std::vector<double> wv, we;
    for_vertices(mg, level, [&](const VertexCL& v) {
        for (size_t d = 0; d < 3; ++d) wv.push_back(v.Unknowns.Exist(id) ? w.Data[v.Unknowns(id) + d * block] : 0.);
    });
    for_edges(mg, level, [&](const EdgeCL& e) {
        for (size_t d = 0; d < 3; ++d) we.push_back(e.Unknowns.Exist(id) ? w.Data[e.Unknowns(id) + d * block] : 0.);
    });
    check(tf_wind_upload(context(), wv.data(), we.data()));
}

void download_matrix(int mat, MatrixCL& out) {
    int64_t rows = 0, nnz = 0;
    check(tf_matrix_info(context(), mat, &rows, &nnz));
    MatrixCL m((size_t)rows, (size_t)rows, (size_t)nnz);
    check(tf_matrix_download(context(), mat, reinterpret_cast<int64_t*>(m.raw_row()),
                             reinterpret_cast<int64_t*>(m.raw_col()), m.raw_val()));
    out = m;
    out.IncrementVersion();
}

}  // namespace

tf_context* context() {
    Session& s = session();
    if (!s.ctx) {
        const int st = tf_create(&s.ctx, 0);
        if (st != TF_OK) {
            s.ctx = nullptr;
            throw DROPSErrCL(std::string("libtracefem: ") + tf_status_string(st));
        }
    }
    return s.ctx;
}

void Invalidate() {
    Session& s = session();
    s.mg = nullptr;
    s.ls_data = nullptr;
}

void SetLoad(int rhs_kind, const std::vector<double>& parameters) {
    session().rhs_kind = rhs_kind;
    session().rhs_par = parameters;
}

FlatLevel Flatten(const MultiGridCL& mg, Uint level) {
    FlatLevel F;
    std::unordered_map<const VertexCL*, int32_t> vid;
    std::unordered_map<const EdgeCL*, int32_t> eid;
    for_vertices(mg, level, [&](const VertexCL& v) {
        vid.emplace(&v, (int32_t)vid.size());
        for (int c = 0; c < 3; ++c) F.coords.push_back(v.GetCoord()[c]);
    });
    for_edges(mg, level, [&](const EdgeCL& e) {
        eid.emplace(&e, (int32_t)eid.size());
        F.edge_v.push_back(vid.at(e.GetVertex(0)));
        F.edge_v.push_back(vid.at(e.GetVertex(1)));
    });
    for_tets(mg, level, [&](const TetraCL& t) {
        for (int i = 0; i < 4; ++i) F.tet_v.push_back(vid.at(t.GetVertex(i)));
        for (int i = 0; i < 6; ++i) F.tet_e.push_back(eid.at(t.GetEdge(i)));
    });
    return F;
}

void LevelSetValues(const MultiGridCL& mg, Uint level, const VecDescCL& ls, std::vector<double>& ls_vert,
                    std::vector<double>& ls_edge) {
    if (!ls.RowIdx || !ls.RowIdx->NumUnknownsEdge())
        throw std::invalid_argument("gpu: the level set must be a P2 VecDescCL");
    const Uint li = ls.RowIdx->GetIdx();
    ls_vert.clear();
    ls_edge.clear();
    for_vertices(mg, level, [&](const VertexCL& v) { ls_vert.push_back(ls.Data[v.Unknowns(li)]); });
    for_edges(mg, level, [&](const EdgeCL& e) { ls_edge.push_back(ls.Data[e.Unknowns(li)]); });
}

size_t DistributeDOFs(IdxDescCL& idx, Uint level, MultiGridCL& mg, VecDescCL const* levelSet, double dist) {
    if (!levelSet) return idx.DistributeDOFs(level, mg, nullptr, dist);  // standard FE numbering: not this path
    ensure_uploaded(mg, level, *levelSet);
    tf_context* c = context();
    const int fe = fe_of(idx);
    int64_t n_active = 0, n = 0;
    check(tf_distribute_dofs(c, fe, dist, &n_active, &n));
    const size_t nv = session().nv, ne = session().ne;
    std::vector<int32_t> dof_vert(nv), dof_edge(fe == TF_P2IF ? ne : 0), active((size_t)std::max<int64_t>(n_active, 1));
    check(tf_dofs_download(c, dof_vert.data(), fe == TF_P2IF ? dof_edge.data() : nullptr, active.data(), nullptr));
    // a fresh index with no unknowns (the old numbering freed, vectors of idx
    // resized to 0): the reference's own call on no active tet
    idx.DistributeDOFs(level, mg, nullptr, -1.);
    const Uint id = idx.GetIdx();
    size_t k = 0, a = 0;
    for (auto it = mg.GetTriangTetraBegin(level); it != mg.GetTriangTetraEnd(level); ++it, ++k)
        if (a < (size_t)n_active && (size_t)active[a] == k) {
            it->Unknowns.Prepare(id);
            it->Unknowns(id) = id;  // marks the tet, as DistributeDOFs does
            ++a;
        }
    k = 0;
    for (auto it = mg.GetTriangVertexBegin(level); it != mg.GetTriangVertexEnd(level); ++it, ++k)
        if (dof_vert[k] >= 0) {
            it->Unknowns.Prepare(id);
            it->Unknowns(id) = (IdxT)dof_vert[k];
        }
    if (fe == TF_P2IF) {
        k = 0;
        for (auto it = mg.GetTriangEdgeBegin(level); it != mg.GetTriangEdgeEnd(level); ++it, ++k)
            if (dof_edge[k] >= 0) {
                it->Unknowns.Prepare(id);
                it->Unknowns(id) = (IdxT)dof_edge[k];
            }
    }
    idx.ChangeNumUnknowns((IdxT)((idx.IsScalar() ? 1 : 3) * n));
    session().idx_id = id;
    session().idx_dist = dist;
    return (size_t)n_active;
}

void setupFESystem(MultiGridCL const& mg, FESystem& system) {
    if (system.matrices.empty() && system.vectors.empty()) return;
    const IdxDescCL& row = system.matrices.empty() ? *system.vectors[0]->RowIdx : *system.matrices[0]->RowIdx;
    const Uint level = row.TriangLevel();
    ensure_uploaded(mg, level, system.params.levelSet);
    tf_context* c = context();
    Session& s = session();
    const int fe = fe_of(row);
    int64_t n_active = 0, n = 0;
    check(tf_distribute_dofs(c, fe, s.idx_id == row.GetIdx() ? s.idx_dist : 0., &n_active, &n));
    if ((IdxT)n != row.NumUnknowns())
        throw DROPSErrCL("gpu::setupFESystem: the row index is not the DistributeDOFs numbering of this level set");
    const auto& ch = system.params.surfCahnHilliardParams;
    unsigned forms = 0;
    std::vector<int> handle(system.matrices.size());
    for (size_t k = 0; k < system.matrices.size(); ++k) {
        const auto f = system.matrices[k]->form;
        int h = -1;
        if (fe == TF_P1IF) {
            if (f == &LocalAssembler::M_P1P1) h = TF_FORM_M;
            else if (f == &LocalAssembler::A_P1P1) h = TF_FORM_A;
            else if (f == &LocalAssembler::C_n_P1P1) h = TF_FORM_CN;
            else if (f == &LocalAssembler::LaplaceM_P1P1) h = TF_FORM_LAPM;
            else if (f == &LocalAssembler::N_P1P1) h = TF_FORM_N;
        } else if (f == &LocalAssembler::M_P2P2) {
            h = TF_FORM_M;
        }
        if (h < 0) throw std::invalid_argument("gpu::setupFESystem: a form this GPU path does not assemble");
        handle[k] = h;
        forms |= 1u << h;
    }
    if (forms & (1u << TF_FORM_LAPM)) {
        if (ch.useDegenerateMobility && !ch.chi) throw std::invalid_argument("buildMobility: chi is nullptr");
        upload_vec(TF_VEC_CHI, ch.useDegenerateMobility ? ch.chi->Data : VectorCL());
    }
    if (forms & (1u << TF_FORM_N)) {
        if (!ch.u_T) throw std::invalid_argument("buildWindCH: u_T is nullptr");
        upload_wind(mg, level, *ch.u_T);
    }
    int rhs = TF_RHS_NONE;
    for (auto* v : system.vectors) {
        if (v->form != &LocalAssembler::F_concentration_P1 || fe != TF_P1IF)
            throw std::invalid_argument("gpu::setupFESystem: a load vector this GPU path does not assemble");
        if (s.rhs_kind == TF_RHS_NONE)
            throw std::invalid_argument("gpu::setupFESystem: F_concentration_P1 needs gpu::SetLoad");
        rhs = s.rhs_kind;
    }
    int64_t nnz = 0;
    check(tf_setup_fe_system(c, forms, rhs, s.rhs_par.empty() ? nullptr : s.rhs_par.data(), (int)s.rhs_par.size(),
                             &nnz));
    for (size_t k = 0; k < system.matrices.size(); ++k) download_matrix(handle[k], system.matrices[k]->Data);
    for (auto* v : system.vectors) {
        v->Data.resize((size_t)n);
        check(tf_vec_download(c, TF_VEC_RHS, Addr(v->Data), n));
    }
}

bool PCGSolverCL::solve(const MatrixCL& A, VectorCL& x, const VectorCL& b) {
    tf_context* c = context();
    check(tf_matrix_upload(c, (int64_t)A.num_rows(), reinterpret_cast<const int64_t*>(A.raw_row()),
                           reinterpret_cast<const int64_t*>(A.raw_col()), A.raw_val()));
    upload_vec(TF_VEC_B, b);
    upload_vec(TF_VEC_X, x);
    int it = maxiter_;
    double res = tol_;
    const int st = tf_pcg_jacobi(c, TF_MAT_USER, TF_VEC_B, TF_VEC_X, precision_, &it, &res, rel_ ? 1 : 0);
    if (st != TF_OK && st != TF_ERR_NOT_CONVERGED) check(st);
    check(tf_vec_download(c, TF_VEC_X, Addr(x), (int64_t)x.size()));
    iter_ = it;
    res_ = res;
    return st == TF_OK;
}

bool GMResSolverCL::solve(const MatrixCL& A, VectorCL& x, const VectorCL& b) {
    tf_context* c = context();
    check(tf_matrix_upload(c, (int64_t)A.num_rows(), reinterpret_cast<const int64_t*>(A.raw_row()),
                           reinterpret_cast<const int64_t*>(A.raw_col()), A.raw_val()));
    upload_vec(TF_VEC_B, b);
    upload_vec(TF_VEC_X, x);
    int it = maxiter_;
    double res = tol_;
    const int st = tf_gmres_jacobi(c, TF_MAT_USER, TF_VEC_B, TF_VEC_X, restart_, 0, precision_, &it, &res, rel_ ? 1 : 0);
    if (st != TF_OK && st != TF_ERR_NOT_CONVERGED) check(st);
    check(tf_vec_download(c, TF_VEC_X, Addr(x), (int64_t)x.size()));
    iter_ = it;
    res_ = res;
    return st == TF_OK;
}

}  // namespace gpu
}  // namespace DROPS
