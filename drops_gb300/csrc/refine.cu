// Narrow-band refinement of a tetrahedral mesh towards the zero level of a
// distance function, with DROPS's refinement algorithm and tet order.
//
// This is the mesh-generation step of the surface Cahn-Hilliard driver
// (surfphasesep/surfphasesep.cpp:170-181): AdapTriangCL::MakeInitialTriang
// (levelset/adaptriang.cpp:36-44, 58-94) with DistMarkingStrategyCL
// (levelset/marking_strategy.cpp:356-398) over MultiGridCL::Refine
// (geom/multigrid.cpp:188-453) and TetraCL's refinement members
// (geom/simplex.cpp:656-997, geom/simplex.tpp:338-376).  The result is the
// last triangulation level (TriangFillCL, geom/multigrid.cpp:1072-1083):
// tets of every level that are unrefined, level by level in list order, then
// the tets of the last level.  DOF numbering and assembly run on that mesh as
// on any uploaded mesh, so the tet order, each tet's vertex order and the
// vertex coordinates must be the reference's bit for bit.
//
// This file is the sequential form: a walk over per-level tet lists whose
// order is the product (children are appended in rule order, removed ones
// leave the list, survivors keep their places), step by step as the
// reference does it.  It serves tf_refine_band (host arrays, no device) and
// generates the refinement rules.  The device path (tf_mesh_refine_band)
// runs the same algorithm as data-parallel passes (refine_par.cu).
//
// Object model (what the order and the marks depend on):
//   vertices  coordinates, level, removal mark;
//   edges     ordered vertex pair (the global orientation of the mesh),
//             level, refinement counter MFR (number of committed regular
//             refinements of tets containing the edge), midvertex, removal
//             mark;
//   tets      vertices and edges in local order, level, parent, children in
//             rule order, refinement rule and mark (NoRef 0, pattern 1..62,
//             regular 63, green-regular 127, remove 64).
// Faces carry no information the order or the marks depend on and are not
// modelled.  Recycle bins are: an edge or tet found again within one
// RefineGrid pass only if it was created or rescued in that pass, looked up
// by its vertex tuple in order, first entry first.
//
// Refinement rules: the 64 edge patterns of a tet, each a list of children
// over the ten local points (vertices 0..3, midpoint 4+e of edge e), are
// generated here: every face with two split edges is cut from the midpoint
// of its lower-numbered split edge to the far end of the other one; the
// interior is the tetrahedrisation of the points that conforms to those face
// triangulations, and where there are several, the one without a diagonal
// between midpoints of opposite edges, else the one with the diagonal 5-8,
// then 4-9, then 6-7.  A child lists its points in the order 0,4,1,5,6,2,7,8,
// 9,3 (every midpoint just before the higher end of its edge, which keeps
// the global edge orientation); children are ordered with the eight regular
// children first, each group lexicographically.  These are the choices of
// geom/triang.cpp and geom/topo.cpp, which the golden fixtures pin.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <unordered_map>
#include <vector>

#include "tf_internal.cuh"

namespace tf {
namespace refine {

constexpr int kVertOfEdge[6][2] = {{0, 1}, {0, 2}, {1, 2}, {0, 3}, {1, 3}, {2, 3}};
constexpr int kFaces[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
constexpr uint16_t kNoRef = 0, kRegRef = 63, kGreenRegRef = 127, kRemove = 64;

struct Rule {
    int nch = 0;
    uint8_t ch[8][4];   // children, local points
    uint64_t edges[2];  // local point pairs used by the children: bit 10 a + b (a < b)
};

// ---- rule generation -------------------------------------------------------
struct RuleGen {
    int P[10][3];  // local points, coordinates doubled
    static int edge_of(int a, int b) {
        if (a > b) std::swap(a, b);
        for (int e = 0; e < 6; ++e)
            if (kVertOfEdge[e][0] == a && kVertOfEdge[e][1] == b) return e;
        return -1;
    }
    RuleGen() {
        const int C[4][3] = {{0, 0, 0}, {2, 0, 0}, {0, 2, 0}, {0, 0, 2}};
        for (int i = 0; i < 4; ++i)
            for (int k = 0; k < 3; ++k) P[i][k] = C[i][k];
        for (int e = 0; e < 6; ++e)
            for (int k = 0; k < 3; ++k) P[4 + e][k] = (C[kVertOfEdge[e][0]][k] + C[kVertOfEdge[e][1]][k]) / 2;
    }
    int64_t vol(int a, int b, int c, int d) const {
        int64_t m[3][3];
        for (int k = 0; k < 3; ++k) {
            m[0][k] = P[b][k] - P[a][k];
            m[1][k] = P[c][k] - P[a][k];
            m[2][k] = P[d][k] - P[a][k];
        }
        return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
               m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    }
    // point p in the closed tet t (nonzero volume)
    bool in_closed(const int t[4], int p) const {
        const int64_t V = vol(t[0], t[1], t[2], t[3]);
        const int64_t s[4] = {vol(p, t[1], t[2], t[3]), vol(t[0], p, t[2], t[3]), vol(t[0], t[1], p, t[3]),
                              vol(t[0], t[1], t[2], p)};
        for (int i = 0; i < 4; ++i)
            if ((V > 0 && s[i] < 0) || (V < 0 && s[i] > 0)) return false;
        return true;
    }
    using Tri = std::array<int, 3>;
    static Tri tri(int a, int b, int c) {
        Tri t{a, b, c};
        std::sort(t.begin(), t.end());
        return t;
    }
    void face_tris(const int f[3], int pat, std::vector<Tri>& out) const {
        const int a = f[0], b = f[1], c = f[2];
        const int es[3][2] = {{a, b}, {a, c}, {b, c}};
        int marked[3][2], nm = 0;
        for (auto& e : es)
            if (pat >> edge_of(e[0], e[1]) & 1) {
                marked[nm][0] = e[0];
                marked[nm][1] = e[1];
                ++nm;
            }
        auto mid = [](int x, int y) { return 4 + edge_of(x, y); };
        if (nm == 0) {
            out.push_back(tri(a, b, c));
        } else if (nm == 3) {
            const int mab = mid(a, b), mac = mid(a, c), mbc = mid(b, c);
            out.push_back(tri(a, mab, mac));
            out.push_back(tri(b, mab, mbc));
            out.push_back(tri(c, mac, mbc));
            out.push_back(tri(mab, mac, mbc));
        } else if (nm == 1) {
            const int m = mid(marked[0][0], marked[0][1]);
            const int o = a + b + c - marked[0][0] - marked[0][1];
            out.push_back(tri(marked[0][0], m, o));
            out.push_back(tri(marked[0][1], m, o));
        } else {
            int *e1 = marked[0], *e2 = marked[1];
            if (edge_of(e1[0], e1[1]) > edge_of(e2[0], e2[1])) std::swap(e1, e2);
            const int com = (e1[0] == e2[0] || e1[0] == e2[1]) ? e1[0] : e1[1];
            const int f1 = e1[0] == com ? e1[1] : e1[0], f2 = e2[0] == com ? e2[1] : e2[0];
            const int m1 = mid(e1[0], e1[1]), m2 = mid(e2[0], e2[1]);
            out.push_back(tri(com, m1, m2));
            out.push_back(tri(m1, f1, f2));
            out.push_back(tri(m1, f2, m2));
        }
    }
    // all tetrahedrisations of the pattern's points conforming to the face triangulations
    void solve(int pat, std::vector<std::vector<std::array<int, 4>>>& sols) const {
        std::vector<int> pts = {0, 1, 2, 3};
        for (int e = 0; e < 6; ++e)
            if (pat >> e & 1) pts.push_back(4 + e);
        std::vector<Tri> bnd;
        for (auto& f : kFaces) face_tris(f, pat, bnd);
        std::sort(bnd.begin(), bnd.end());
        std::vector<std::array<int, 4>> cand;
        const int np = (int)pts.size();
        for (int i = 0; i < np; ++i)
            for (int j = i + 1; j < np; ++j)
                for (int k = j + 1; k < np; ++k)
                    for (int l = k + 1; l < np; ++l) {
                        const int t[4] = {pts[i], pts[j], pts[k], pts[l]};
                        if (vol(t[0], t[1], t[2], t[3]) == 0) continue;
                        bool ok = true;
                        for (int p : pts)
                            if (p != t[0] && p != t[1] && p != t[2] && p != t[3] && in_closed(t, p)) ok = false;
                        if (ok) cand.push_back({t[0], t[1], t[2], t[3]});
                    }
        const int64_t V = std::llabs(vol(0, 1, 2, 3));
        std::vector<std::array<int, 4>> chosen;
        std::vector<Tri> front(bnd);
        rec(cand, bnd, chosen, front, 0, V, sols);
    }
    void rec(const std::vector<std::array<int, 4>>& cand, const std::vector<Tri>& bnd,
             std::vector<std::array<int, 4>>& chosen, std::vector<Tri>& front, int64_t vs, int64_t V,
             std::vector<std::vector<std::array<int, 4>>>& sols) const {
        if (vs == V) {
            if (front.empty()) {
                auto s = chosen;
                std::sort(s.begin(), s.end());
                if (std::find(sols.begin(), sols.end(), s) == sols.end()) sols.push_back(s);
            }
            return;
        }
        if (front.empty()) return;
        const Tri f = *std::min_element(front.begin(), front.end());
        for (const auto& t : cand) {
            if (std::find(chosen.begin(), chosen.end(), t) != chosen.end()) continue;
            int hit = 0;
            for (int q : f)
                for (int x : t) hit += q == x;
            if (hit != 3) continue;
            std::vector<Tri> nf(front);
            bool ok = true;
            for (int o = 0; o < 4 && ok; ++o) {
                int g[3], k = 0;
                for (int i = 0; i < 4; ++i)
                    if (i != o) g[k++] = t[i];
                const Tri gt = tri(g[0], g[1], g[2]);
                auto it = std::find(nf.begin(), nf.end(), gt);
                if (it != nf.end())
                    nf.erase(it);
                else if (std::binary_search(bnd.begin(), bnd.end(), gt))
                    ok = false;
                else
                    nf.push_back(gt);
            }
            const int64_t nv = vs + std::llabs(vol(t[0], t[1], t[2], t[3]));
            if (!ok || nv > V) continue;
            chosen.push_back(t);
            rec(cand, bnd, chosen, nf, nv, V, sols);
            chosen.pop_back();
        }
    }
};

struct Tables {
    Rule rule[64];
    bool ok = false;
};

static int rank_of(int p) {
    static const int r[10] = {0, 2, 5, 9, 1, 3, 4, 6, 7, 8};
    return r[p];
}

static const Tables& tables() {
    static Tables T = [] {
        Tables t;
        RuleGen G;
        std::vector<std::array<int, 4>> regular;
        std::vector<std::vector<std::array<int, 4>>> sols_all[64];
        bool ok = true;
        for (int pat = 0; pat < 64; ++pat) {
            auto& sols = sols_all[pat];
            G.solve(pat, sols);
            if (sols.empty()) ok = false;
        }
        // the choice among several tetrahedrisations
        auto score = [](const std::vector<std::array<int, 4>>& s) {
            auto has = [&](int a, int b) {
                for (auto& t : s) {
                    bool ia = false, ib = false;
                    for (int x : t) ia |= x == a, ib |= x == b;
                    if (ia && ib) return true;
                }
                return false;
            };
            return (has(5, 8) ? 1 : 0) + (has(4, 9) ? 2 : 0) + (has(6, 7) ? 4 : 0);
        };
        std::vector<std::array<int, 4>> pick[64];
        for (int pat = 0; pat < 64 && ok; ++pat) {
            auto& sols = sols_all[pat];
            int best = -1, bs = 1 << 30;
            for (int i = 0; i < (int)sols.size(); ++i) {
                const int s = score(sols[i]);
                if (s < bs) bs = s, best = i;
            }
            pick[pat] = sols[best];
            for (auto& c : pick[pat]) std::sort(c.begin(), c.end(), [](int a, int b) { return rank_of(a) < rank_of(b); });
        }
        if (ok) {
            regular = pick[63];
            std::sort(regular.begin(), regular.end());
            for (int pat = 0; pat < 64; ++pat) {
                auto ch = pick[pat];
                std::sort(ch.begin(), ch.end(), [&](const std::array<int, 4>& a, const std::array<int, 4>& b) {
                    const bool ra = std::binary_search(regular.begin(), regular.end(), a);
                    const bool rb = std::binary_search(regular.begin(), regular.end(), b);
                    if (ra != rb) return ra;
                    return a < b;
                });
                Rule& R = t.rule[pat];
                R.nch = (int)ch.size();
                R.edges[0] = R.edges[1] = 0;
                if (R.nch > 8) ok = false;
                for (int i = 0; i < R.nch && i < 8; ++i) {
                    for (int k = 0; k < 4; ++k) R.ch[i][k] = (uint8_t)ch[i][k];
                    for (int e = 0; e < 6; ++e) {
                        int a = ch[i][kVertOfEdge[e][0]], b = ch[i][kVertOfEdge[e][1]];
                        if (a > b) std::swap(a, b);
                        const int bit = 10 * a + b;
                        R.edges[bit >> 6] |= 1ull << (bit & 63);
                    }
                }
            }
        }
        t.ok = ok;
        return t;
    }();
    return T;
}

// ---- the multilevel mesh ----------------------------------------------------
struct Vtx {
    double x[3];
    int level;
    bool rm;
};
struct Edge {
    int v[2];
    int level;
    int mfr;
    int mid;
    bool rm;
};
struct Tet {
    int v[4];
    int e[6];
    int level;
    int parent;
    int child[8];
    int nch;
    uint16_t rule, mark;
};

static uint64_t key2(int a, int b) { return (uint64_t)(uint32_t)a << 32 | (uint32_t)b; }
struct Key4 {
    int v[4];
    bool operator==(const Key4& o) const { return std::memcmp(v, o.v, sizeof v) == 0; }
};
struct Key4Hash {
    size_t operator()(const Key4& k) const {
        uint64_t h = 1469598103934665603ull;
        for (int x : k.v) h = (h ^ (uint32_t)x) * 1099511628211ull;
        return (size_t)h;
    }
};

using DistFn = double (*)(const double*, const double[3]);

struct MG {
    std::vector<Vtx> V;
    std::vector<Edge> E;
    std::vector<Tet> T;
    std::vector<std::vector<int>> tl, el, vl;  // per-level lists (list order)
    std::unordered_map<uint64_t, int> ebin;
    std::unordered_map<Key4, int, Key4Hash> tbin;
    const Tables* tab = nullptr;
    int err = 0;

    int last() const { return (int)tl.size() - 1; }
    void append_level() {
        tl.emplace_back();
        el.emplace_back();
        vl.emplace_back();
    }
    int make_vertex(const double x[3], int level) {
        Vtx v;
        for (int k = 0; k < 3; ++k) v.x[k] = x[k];
        v.level = level;
        v.rm = false;
        V.push_back(v);
        vl[level].push_back((int)V.size() - 1);
        return (int)V.size() - 1;
    }
    int make_edge(int a, int b, int level) {
        Edge e;
        e.v[0] = a;
        e.v[1] = b;
        e.level = level;
        e.mfr = 0;
        e.mid = -1;
        e.rm = false;
        E.push_back(e);
        el[level].push_back((int)E.size() - 1);
        return (int)E.size() - 1;
    }
    int make_tet(const int v[4], int parent) {
        Tet t;
        for (int k = 0; k < 4; ++k) t.v[k] = v[k];
        for (int k = 0; k < 6; ++k) t.e[k] = -1;
        t.level = parent < 0 ? 0 : T[parent].level + 1;
        t.parent = parent;
        t.nch = 0;
        t.rule = kNoRef;
        t.mark = kNoRef;
        T.push_back(t);
        tl[t.level].push_back((int)T.size() - 1);
        return (int)T.size() - 1;
    }
    void recycle_edge(int e) { ebin.emplace(key2(E[e].v[0], E[e].v[1]), e); }
    int find_edge(int a, int b) const {
        auto it = ebin.find(key2(a, b));
        return it == ebin.end() ? -1 : it->second;
    }
    void clear_bins() {
        ebin.clear();
        tbin.clear();
    }

    bool is_regular(const Tet& t) const { return t.level == 0 || T[t.parent].rule == kRegRef; }
    static bool marked_for_ref(const Tet& t) { return t.mark != kNoRef && t.mark != kRemove; }
    void commit(const Tet& t) {
        for (int e : t.e) ++E[e].mfr;
    }
    void uncommit(const Tet& t) {
        for (int e : t.e) --E[e].mfr;
    }
    // local point i of tet t: vertex, or the midvertex of edge i - 4
    int vert_mid(const Tet& t, int i) const { return i < 4 ? t.v[i] : E[t.e[i - 4]].mid; }

    // TetraCL::RestrictMark (geom/simplex.cpp:770-834)
    void restrict_mark(int ti) {
        Tet& t = T[ti];
        if (t.rule == kNoRef) {
            if (t.mark == kRegRef && is_regular(t)) commit(t);
            if (t.level == 0 && t.mark == kRemove) t.mark = kNoRef;
        } else if (t.rule == kRegRef) {
            bool keep = false;
            for (int c = 0; c < t.nch; ++c) {
                Tet& ch = T[t.child[c]];
                if (ch.mark == kRemove)
                    ch.mark = kNoRef;
                else
                    keep = true;
            }
            if (!keep) {
                t.mark = kNoRef;
                uncommit(t);
            }
        } else {
            bool reg = false;
            for (int c = 0; c < t.nch; ++c) {
                Tet& ch = T[t.child[c]];
                if (!reg) {
                    if (marked_for_ref(ch)) {
                        reg = true;
                    } else {
                        for (int e : ch.e)
                            if (E[e].mfr && E[e].level != t.level) {
                                reg = true;
                                break;
                            }
                    }
                }
                ch.mark = kNoRef;
            }
            if (reg) {
                t.mark = kRegRef;
                commit(t);
            } else {
                t.mark = kNoRef;
            }
        }
    }
    // TetraCL::Close (geom/simplex.tpp:351-376)
    void close(Tet& t) {
        unsigned m = 0;
        for (int j = 0; j < 6; ++j)
            if (E[t.e[j]].mfr) m |= 1u << j;
        if (m == kRegRef)
            t.mark = kGreenRegRef;
        else if (m == kNoRef) {
            if (t.mark != kRemove) t.mark = kNoRef;
        } else
            t.mark = (uint16_t)m;
    }
    void close_grid(int L) {
        for (int ti : tl[L]) {
            Tet& t = T[ti];
            if (is_regular(t) && t.mark != kRegRef) close(t);
        }
    }
    // TetraCL::ClearAllRemoveMarks (geom/simplex.cpp:749-768)
    void clear_all_remove_marks(const Tet& t) {
        for (int c = 0; c < t.nch; ++c) {
            const Tet& ch = T[t.child[c]];
            for (int v : ch.v) V[v].rm = false;
            for (int e : ch.e) E[e].rm = false;
        }
    }
    static bool rule_has_edge(const Rule& R, int a, int b) {
        if (a > b) std::swap(a, b);
        const int bit = 10 * a + b;
        return R.edges[bit >> 6] >> (bit & 63) & 1;
    }
    // TetraCL::RecycleReusables (geom/simplex.cpp:656-747)
    void recycle_reusables(int ti) {
        const Tet& t = T[ti];
        const Rule& my = tab->rule[t.rule & 63];
        const Rule& nw = tab->rule[t.mark & 63];
        uint64_t common[2] = {my.edges[0] & nw.edges[0], my.edges[1] & nw.edges[1]};
        for (int c = 0; c < my.nch; ++c) {
            const Tet& ch = T[t.child[c]];
            for (int j = 0; j < 6; ++j) {
                int a = my.ch[c][kVertOfEdge[j][0]], b = my.ch[c][kVertOfEdge[j][1]];
                if (a < 4 && b < 4) continue;  // an edge of the parent
                if (a > b) std::swap(a, b);
                const int bit = 10 * a + b;
                if (common[bit >> 6] >> (bit & 63) & 1) {
                    V[ch.v[kVertOfEdge[j][0]]].rm = false;
                    V[ch.v[kVertOfEdge[j][1]]].rm = false;
                    E[ch.e[j]].rm = false;
                    recycle_edge(ch.e[j]);
                    common[bit >> 6] &= ~(1ull << (bit & 63));
                }
            }
        }
        for (int c = 0; c < my.nch; ++c) {
            bool in_new = false;
            for (int d = 0; d < nw.nch && !in_new; ++d) in_new = std::memcmp(my.ch[c], nw.ch[d], 4) == 0;
            if (in_new) {
                Tet& ch = T[t.child[c]];
                ch.mark = kNoRef;
                Key4 k{{ch.v[0], ch.v[1], ch.v[2], ch.v[3]}};
                tbin.emplace(k, t.child[c]);
            }
        }
    }
    // MultiGridCL::UnrefineGrid (geom/multigrid.cpp:223-331, serial branch)
    void unrefine_grid(int L) {
        const int nl = L + 1;
        for (int v : vl[nl]) V[v].rm = true;
        for (int e : el[nl]) E[e].rm = true;
        for (int ti : tl[L]) {
            Tet& t = T[ti];
            if (t.rule == kNoRef) continue;
            if (t.mark == t.rule) {
                clear_all_remove_marks(t);
            } else {
                for (int c = 0; c < t.nch; ++c) T[t.child[c]].mark = kRemove;
                if (t.mark != kNoRef) recycle_reusables(ti);
            }
        }
        std::vector<int>& lst = tl[nl];
        lst.erase(std::remove_if(lst.begin(), lst.end(), [&](int ti) { return T[ti].mark == kRemove; }), lst.end());
        for (int e : el[L])
            if (E[e].mid >= 0 && V[E[e].mid].rm) E[e].mid = -1;
        vl[nl].erase(std::remove_if(vl[nl].begin(), vl[nl].end(), [&](int v) { return V[v].rm; }), vl[nl].end());
        el[nl].erase(std::remove_if(el[nl].begin(), el[nl].end(), [&](int e) { return E[e].rm; }), el[nl].end());
    }
    // TetraCL::CollectEdges + CollectAndLinkChildren (geom/simplex.cpp:836-915, 966-997)
    void refine_tet(int ti) {
        const Rule& R = tab->rule[T[ti].rule & 63];
        int loc[10][10];  // edge object per pair of local points
        for (auto& r : loc)
            for (int& x : r) x = -1;
        for (int j = 0; j < 6; ++j) {
            const int a = kVertOfEdge[j][0], b = kVertOfEdge[j][1];
            const int ei = T[ti].e[j];
            if (E[ei].mfr) {
                const int va = T[ti].v[a], vb = T[ti].v[b];
                int s0, s1;
                if (E[ei].mid >= 0) {
                    s0 = find_edge(va, E[ei].mid);
                    s1 = find_edge(E[ei].mid, vb);
                    if (s0 < 0 || s1 < 0) {
                        err = 1;
                        return;
                    }
                } else {
                    // EdgeCL::BuildSubEdges / BuildMidVertex (geom/simplex.cpp:116-161, simplex.tpp:169-174)
                    const Edge ed = E[ei];
                    double m[3];
                    for (int k = 0; k < 3; ++k) m[k] = 0.5 * (V[ed.v[0]].x[k] + V[ed.v[1]].x[k]);
                    if ((int)vl.size() <= ed.level + 1) append_level();
                    const int mv = make_vertex(m, ed.level + 1);
                    E[ei].mid = mv;
                    s0 = make_edge(ed.v[0], mv, ed.level + 1);
                    s1 = make_edge(mv, ed.v[1], ed.level + 1);
                    recycle_edge(s0);
                    recycle_edge(s1);
                }
                loc[a][4 + j] = loc[4 + j][a] = s0;
                loc[4 + j][b] = loc[b][4 + j] = s1;
            } else {
                loc[a][b] = loc[b][a] = ei;
            }
        }
        const int nl = T[ti].level + 1;
        // inner edges, in the order of their local point pairs (every one joins a midpoint)
        for (int a = 0; a < 10; ++a)
            for (int b = a + 1; b < 10; ++b) {
                if (!rule_has_edge(R, a, b) || loc[a][b] >= 0) continue;
                int p = a, q = b;
                if (rank_of(p) > rank_of(q)) std::swap(p, q);
                const int vp = vert_mid(T[ti], p), vq = vert_mid(T[ti], q);
                int ei = find_edge(vp, vq);
                if (ei < 0) {
                    ei = make_edge(vp, vq, nl);
                    recycle_edge(ei);
                }
                loc[a][b] = loc[b][a] = ei;
            }
        T[ti].nch = R.nch;
        for (int c = 0; c < R.nch; ++c) {
            int cv[4];
            for (int k = 0; k < 4; ++k) cv[k] = vert_mid(T[ti], R.ch[c][k]);
            Key4 key{{cv[0], cv[1], cv[2], cv[3]}};
            auto it = tbin.find(key);
            const int ci = it != tbin.end() ? it->second : make_tet(cv, ti);
            T[ti].child[c] = ci;
            for (int j = 0; j < 6; ++j) T[ci].e[j] = loc[R.ch[c][kVertOfEdge[j][0]]][R.ch[c][kVertOfEdge[j][1]]];
        }
    }
    // MultiGridCL::RefineGrid (geom/multigrid.cpp:334-386, serial branch)
    void refine_grid(int L) {
        if (L == last()) append_level();
        const std::vector<int> lst = tl[L];
        for (int ti : lst) {
            Tet& t = T[ti];
            if (t.mark == t.rule) continue;
            if (t.mark == kRemove) {
                err = 2;
                return;
            }
            t.rule = t.mark;
            if (t.mark == kNoRef)
                t.nch = 0;
            else
                refine_tet(ti);
            if (err) return;
        }
        clear_bins();
    }
    // MultiGridCL::Refine (geom/multigrid.cpp:389-453, serial branch; no periodic edges)
    void refine() {
        const int top = last();
        for (int L = top; L >= 0; --L) {
            for (int ti : tl[L]) restrict_mark(ti);
            close_grid(L);
        }
        for (int L = 0; L <= top && !err; ++L) {
            if (tl[L].empty()) continue;
            if (L) close_grid(L);
            if (L != top) unrefine_grid(L);
            refine_grid(L);
        }
        while (tl.size() > 1 && tl.back().empty()) {
            tl.pop_back();
            el.pop_back();
            vl.pop_back();
        }
        clear_bins();
    }
    // TetraCL::IsInTriang for the last level, in TriangFillCL order
    template <class F>
    void for_triang(F&& f) const {
        const int L = last();
        for (int l = 0; l <= L; ++l)
            for (int ti : tl[l])
                if (l == L || T[ti].rule == kNoRef) f(ti);
    }
    // DistMarkingStrategyCL::visit (levelset/marking_strategy.cpp:356-398) over the triangulation
    bool mark(DistFn dist, const double* par, double width, int clevel, int flevel) {
        bool modified = false;
        for_triang([&](int ti) {
            Tet& t = T[ti];
            double d = std::numeric_limits<double>::max();
            int npos = 0;
            for (int j = 0; j < 4; ++j) {
                const double v = dist(par, V[t.v[j]].x);
                if (v >= 0) ++npos;
                d = std::min(d, std::fabs(v));
            }
            for (int j = 0; j < 6; ++j) {
                const Edge& e = E[t.e[j]];
                double x[3];
                for (int k = 0; k < 3; ++k) x[k] = (V[e.v[0]].x[k] + V[e.v[1]].x[k]) * 0.5;
                const double v = dist(par, x);
                if (v >= 0) ++npos;
                d = std::min(d, std::fabs(v));
            }
            double b[3];
            for (int k = 0; k < 3; ++k)
                b[k] = 0.25 * (((V[t.v[0]].x[k] + V[t.v[1]].x[k]) + V[t.v[2]].x[k]) + V[t.v[3]].x[k]);
            d = std::min(d, std::fabs(dist(par, b)));
            const bool change = npos != 0 && npos != 10;
            const int l = t.level;
            const int want = (d <= width || change) ? flevel : clevel;
            if (l < want || (l == want && !is_regular(t))) {
                t.mark = kRegRef;
                modified = true;
            } else if (l > want) {
                t.mark = kRemove;
                modified = true;
            }
        });
        return modified;
    }
};

// distance functions, the same expressions as the device level sets
static double nrm3(double a, double b, double c) { return std::sqrt(a * a + b * b + c * c); }
static double dist_sphere(const double* p, const double x[3]) {
    return nrm3(x[0] - p[0], x[1] - p[1], x[2] - p[2]) - p[3];
}
static double dist_torus(const double* p, const double x[3]) {
    const int ax = (int)p[2];
    const int a0 = (ax + 1) % 3, a1 = (ax + 2) % 3;
    const double rho = std::sqrt(x[a0] * x[a0] + x[a1] * x[a1]) - p[0];
    return std::sqrt(rho * rho + x[ax] * x[ax]) - p[1];
}
static double dist_plane(const double* p, const double x[3]) { return ((p[0] * x[0] + p[1] * x[1]) + p[2] * x[2]) - p[3]; }

}  // namespace refine

// Runs MakeInitialTriang on the mesh (coords, tet_v): a mesh whose tets list
// their vertices in one global order (as BrickBuilderCL's do).
int refine_band(int64_t nv, const double* coords, int64_t nt, const int32_t* tet_v, int kind, const double* par,
                int npar, double width, int clevel, int flevel, RefinedMesh& out) {
    using namespace refine;
    DistFn fn = nullptr;
    int need = 0;
    switch (kind) {
        case TF_LS_SPHERE: fn = dist_sphere; need = 4; break;
        case TF_LS_TORUS: fn = dist_torus; need = 3; break;
        case TF_LS_PLANE: fn = dist_plane; need = 4; break;
        default: return TF_ERR_BAD_INPUT;
    }
    if (npar < need || !par || nv <= 0 || nt <= 0 || !coords || !tet_v) return TF_ERR_BAD_INPUT;
    if (clevel < 0 || flevel < clevel || flevel > 30 || !(width >= 0)) return TF_ERR_BAD_INPUT;
    if (kind == TF_LS_TORUS && (par[2] < 0 || par[2] > 2)) return TF_ERR_BAD_INPUT;
    for (int64_t i = 0; i < 4 * nt; ++i)
        if (tet_v[i] < 0 || tet_v[i] >= nv) return TF_ERR_BAD_INPUT;
    const Tables& tab = tables();
    if (!tab.ok) return TF_ERR_INTERNAL;
    MG g;
    g.tab = &tab;
    g.append_level();
    g.V.reserve((size_t)nv * 4);
    for (int64_t v = 0; v < nv; ++v) g.make_vertex(coords + 3 * v, 0);
    // TetraCL::BuildEdges per tet in order (geom/simplex.cpp:568-605).  An
    // edge met in both directions means the tets do not share one vertex
    // order, which the refinement's edge lookups rely on: refused.
    for (int64_t t = 0; t < nt; ++t) {
        const int ti = g.make_tet(tet_v + 4 * t, -1);
        for (int j = 0; j < 6; ++j) {
            const int a = g.T[ti].v[kVertOfEdge[j][0]], b = g.T[ti].v[kVertOfEdge[j][1]];
            if (a == b || g.find_edge(b, a) >= 0) return TF_ERR_BAD_INPUT;
            int e = g.find_edge(a, b);
            if (e < 0) {
                e = g.make_edge(a, b, 0);
                g.recycle_edge(e);
            }
            g.T[ti].e[j] = e;
        }
    }
    g.clear_bins();
    // AdapTriangCL::MakeInitialTriang (levelset/adaptriang.cpp:36-44): at most
    // 2 * fine level steps, each marking and refining
    double p[16] = {0};
    for (int i = 0; i < npar && i < 16; ++i) p[i] = par[i];
    bool modified = true;
    int steps = 0;
    for (int i = 0; i < 2 * flevel && modified; ++i) {
        modified = g.mark(fn, p, width, clevel, flevel);
        g.refine();
        ++steps;
        if (g.err) return g.err == 1 ? TF_ERR_BAD_INPUT : TF_ERR_INTERNAL;
    }
    // the last triangulation level, vertices and edges numbered by first touch
    std::vector<int32_t> vid(g.V.size(), -1), eid(g.E.size(), -1);
    out = RefinedMesh{};
    out.last_level = g.last();
    out.steps = steps;
    for (auto& l : g.tl) out.per_level.push_back((int64_t)l.size());
    g.for_triang([&](int ti) {
        const Tet& t = g.T[ti];
        for (int v : t.v) {
            if (vid[v] < 0) {
                vid[v] = (int32_t)(out.coords.size() / 3);
                for (int k = 0; k < 3; ++k) out.coords.push_back(g.V[v].x[k]);
            }
            out.tet_v.push_back(vid[v]);
        }
        for (int e : t.e) {
            if (eid[e] < 0) {
                eid[e] = (int32_t)(out.edge_v.size() / 2);
                out.edge_v.push_back(vid[g.E[e].v[0]]);
                out.edge_v.push_back(vid[g.E[e].v[1]]);
            }
            out.tet_e.push_back(eid[e]);
        }
        out.tet_level.push_back(t.level);
    });
    if (out.coords.size() / 3 > (size_t)INT32_MAX || out.edge_v.size() / 2 > (size_t)INT32_MAX) return TF_ERR_CAPACITY;
    return TF_OK;
}

}  // namespace tf

// ---- C ABI ------------------------------------------------------------------
struct tf_refined {
    tf::RefinedMesh m;
};

extern "C" {

int tf_refine_band(int64_t nv, const double* coords, int64_t nt, const int32_t* tet_v, int kind, const double* par,
                   int npar, double width, int coarse_level, int fine_level, tf_refined** out) {
    if (!out) return TF_ERR_BAD_INPUT;
    *out = nullptr;
    tf_refined* r = new tf_refined;
    const int st = tf::refine_band(nv, coords, nt, tet_v, kind, par, npar, width, coarse_level, fine_level, r->m);
    if (st != TF_OK) {
        delete r;
        return st;
    }
    *out = r;
    return TF_OK;
}

int tf_refined_info(const tf_refined* r, int64_t* nv, int64_t* ne, int64_t* nt, int* last_level, int* steps) {
    if (!r) return TF_ERR_BAD_INPUT;
    if (nv) *nv = (int64_t)(r->m.coords.size() / 3);
    if (ne) *ne = (int64_t)(r->m.edge_v.size() / 2);
    if (nt) *nt = (int64_t)r->m.tet_level.size();
    if (last_level) *last_level = r->m.last_level;
    if (steps) *steps = r->m.steps;
    return TF_OK;
}

int tf_refined_get(const tf_refined* r, double* coords, int32_t* tet_v, int32_t* tet_e, int32_t* edge_v,
                   int32_t* tet_level, int64_t* tets_per_level) {
    if (!r) return TF_ERR_BAD_INPUT;
    const tf::RefinedMesh& m = r->m;
    if (coords) std::memcpy(coords, m.coords.data(), sizeof(double) * m.coords.size());
    if (tet_v) std::memcpy(tet_v, m.tet_v.data(), sizeof(int32_t) * m.tet_v.size());
    if (tet_e) std::memcpy(tet_e, m.tet_e.data(), sizeof(int32_t) * m.tet_e.size());
    if (edge_v) std::memcpy(edge_v, m.edge_v.data(), sizeof(int32_t) * m.edge_v.size());
    if (tet_level) std::memcpy(tet_level, m.tet_level.data(), sizeof(int32_t) * m.tet_level.size());
    if (tets_per_level) std::memcpy(tets_per_level, m.per_level.data(), sizeof(int64_t) * m.per_level.size());
    return TF_OK;
}

void tf_refined_free(tf_refined* r) { delete r; }

// The device engine's kernel bodies run as host loops, for checking them
// against the reference's fixtures without a device (not part of the header).
int tf_refine_band_parallel_host(int64_t nv, const double* coords, int64_t nt, const int32_t* tet_v, int kind,
                                 const double* par, int npar, double width, int coarse_level, int fine_level,
                                 tf_refined** out) {
    if (!out) return TF_ERR_BAD_INPUT;
    *out = nullptr;
    tf_refined* r = new tf_refined;
    const int st = tf::refine_band_parallel_host(nv, coords, nt, tet_v, kind, par, npar, width, coarse_level,
                                                 fine_level, r->m);
    if (st != TF_OK) {
        delete r;
        return st;
    }
    *out = r;
    return TF_OK;
}

int tf_refine_rules(int32_t* nch, int32_t* children) {
    const tf::refine::Tables& T = tf::refine::tables();
    if (!T.ok) return TF_ERR_INTERNAL;
    for (int p = 0; p < 64; ++p) {
        if (nch) nch[p] = T.rule[p].nch;
        if (children)
            for (int c = 0; c < 8; ++c)
                for (int k = 0; k < 4; ++k) children[(p * 8 + c) * 4 + k] = c < T.rule[p].nch ? T.rule[p].ch[c][k] : -1;
    }
    return TF_OK;
}

}  // extern "C"
