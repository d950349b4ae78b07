// Surface forms M, A, C_n and the load vector in pair arithmetic (ff.cuh).
//
// The FP64 kernels k_assemble<NL> keep the FP64 pipe 85% busy: per quadrature
// point ~190 FP64 operations for the P2 basis and ~220 lane FMAs for the M and
// A sums, and GB300 issues FP64 at 1/64 of the FP32 rate.  These kernels keep
// the per-tet work in FP64 (GetTrafoTr, the lattice patch with its cut points
// and facet areas: the same code as k_assemble), split the per-tet results
// into float pairs, and run everything per point -- quadrature node, weight
// and its square root, the level-set normal, the projected gradients, the
// load function -- and the element sums on the FP32 pipe in pair arithmetic.
// The sums are formed in the FP64 kernels' point order and point groups; the
// results differ from them by rounding (pair arithmetic carries ~48
// significant bits), inside the 1e-12 row-scaled parity bound.  Covered: M, A,
// C_n (P1 and P2) and a constant or TF_RHS_SPHERE_XYZ load vector; LaplaceM
// and N_P1P1 run k_assemble<4>.  (Pair arithmetic for the per-tet work as
// well was measured slower: the cut points and facet areas then take more
// issue slots on few lanes than their FP64 form takes on the FP64 pipe.)

struct TablesFF {
    ff q2_node[7][3], q2_w[7];
    ff q3_node[15][4], q3_sw[15];
};
__constant__ TablesFF cTF;
static bool g_tables_ff_ready[64] = {false};

static ff host_split(double x) {
    const float h = (float)x;
    return ff{h, (float)(x - (double)h)};
}

static int ensure_tables_ff(Context* c) {
    if (c->device >= 0 && c->device < 64 && g_tables_ff_ready[c->device]) return TF_OK;
    Tables T;
    build_tables(T);
    TablesFF F;
    for (int i = 0; i < 7; ++i) {
        for (int j = 0; j < 3; ++j) F.q2_node[i][j] = host_split(T.q2_node[i][j]);
        F.q2_w[i] = host_split(T.q2_w[i]);
    }
    for (int i = 0; i < 15; ++i) {
        for (int j = 0; j < 4; ++j) F.q3_node[i][j] = host_split(T.q3_node[i][j]);
        F.q3_sw[i] = host_split(T.q3_sw[i]);
    }
    TF_CUDA(c, cudaMemcpyToSymbol(cTF, &F, sizeof(TablesFF)));
    if (c->device >= 0 && c->device < 64) g_tables_ff_ready[c->device] = true;
    return TF_OK;
}

// Per warp.  The FP64 per-tet scratch (geometry, patch) is dead once split
// into pairs, so it shares storage with the point rows.  Point rows are padded
// to an odd number of pairs per lane (11 and 31): a lane's row starts 22 or 62
// words after its neighbour's, so the lanes' 64-bit stores of one column fall
// in distinct banks, and the contraction's reads of one row (one point, ten
// columns) do too.
struct AsmPairFp64 {
    TetGeom g;
    double gM[9], gC[9];
    double ls10[10];
    PatchSmem P;
};
struct AsmPairPts {
    ff phi[32][11];  // sqrt(w) phi_i; n . grad(phi_i) sqrt(w) for the volume rule
    ff sg[32][31];   // [3 i + c]: sqrt(w) (I - n n^T) grad(phi_i)
};
struct AsmPairSmem {
    union {
        AsmPairFp64 d;
        AsmPairPts p;
    } u;
    ff gl[4][3], G[4][3], X[4][3], absdet;
    ff fb[16][3][4], fw[16];
    ff fx[32];  // sqrt(w) f(x_p)
};

// the unit normal grad(phi_h) / |grad(phi_h)| at barycentric b
__device__ __noinline__ void ff_normal(const AsmPairSmem& S, const ff b[4], ff n[3]) {
    ff v[3];
    for (int r = 0; r < 3; ++r) {
        v[r] = ff_mul(b[0], S.G[0][r]);
        for (int k = 1; k < 4; ++k) v[r] = ff_fma(b[k], S.G[k][r], v[r]);
    }
    const ff nn = ff_fma(v[2], v[2], ff_fma(v[1], v[1], ff_mul(v[0], v[0])));
    const ff inv = ff_rsqrt(nn);
    for (int r = 0; r < 3; ++r) n[r] = ff_mul(v[r], inv);
}

__device__ __forceinline__ ff ff_dot3(const ff a[3], const ff b[3]) {
    return ff_fma(a[2], b[2], ff_fma(a[1], b[1], ff_mul(a[0], b[0])));
}

// TF_RHS_SPHERE_XYZ: c * y0 y1 y2 at the closest point y of the sphere
__device__ __noinline__ ff ff_rhs(const RhsPar& R, const ff x[3]) {
    if (R.kind == TF_RHS_CONST) return ff_split(R.p[0]);
    if (R.kind != TF_RHS_SPHERE_XYZ) return ff_of(0.f);
    ff d[3];
    for (int r = 0; r < 3; ++r) d[r] = ff_sub(x[r], ff_split(R.p[r]));
    const ff n2 = ff_dot3(d, d);
    const ff inv = ff_rsqrt(n2);
    const ff dist = ff_sub(ff_mul(n2, inv), ff_split(R.p[3]));
    const ff s = ff_mul(dist, inv);
    ff y[3];
    for (int r = 0; r < 3; ++r) y[r] = ff_sub(x[r], ff_mul(s, d[r]));
    return ff_mul(ff_mul(ff_mul(ff_split(R.p[4]), y[0]), y[1]), y[2]);
}

// The pair forms' per-tet data, one thread per tet: the tet geometry
// (GetTrafoTr and the level set's vertex gradients), the patch on the
// order-2 lattice and (P1, LIN) the linear-level-set test and its constants,
// with the arithmetic of warp_tet_geometry, warp_patch and the P1 kernel's
// linear path done serially.  The FP64 work of a tet is then one thread's
// instead of a warp's with 4 to 25 lanes active, so that every FP64 warp
// instruction works for 32 tets (GB300 runs FP64 at 1/64 of the FP32 rate).
struct TetPrep {
    ff gl[4][3], G[4][3], X[4][3];
    ff fb[16][3][4], fw[16];
    double lin_sg[4][3], lin_G[10], lin_dn[4];
    double absdet;
    ff absdet_ff;
    int nf, lin;
};
constexpr int64_t kPrepChunk = 1 << 18;  // tets per prep pass (about 0.6 GB of records)

template <bool LIN>
__global__ void __launch_bounds__(128) k_prep_tets(AsmArgs A) {
    TetPrep* const out = reinterpret_cast<TetPrep*>(A.prep);
    const int64_t n = A.c1 - A.c0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = A.c0 + (A.prep_order ? A.prep_order[i] : i);
        TetPrep& Q = out[r - A.c0];
        const int32_t t = A.active[r];
        int32_t v[4], e[6];
        mesh_tet(A.M, t, v, e);
        TetGeom g;
        double ls10[10];
        for (int k = 0; k < 4; ++k) {
            mesh_coord(A.M, v[k], g.X[k]);
            ls10[k] = A.lsv[v[k]];
        }
        for (int k = 0; k < 6; ++k) ls10[4 + k] = A.lse[e[k]];
        // warp_tet_geometry, lane by lane
        double Ms[9], Cs[9];
        for (int l = 0; l < 9; ++l) {
            const int rr = l / 3, c = l % 3;
            Ms[l] = g.X[c + 1][rr] - g.X[0][rr];
        }
        for (int l = 0; l < 9; ++l) {
            const int rr = l / 3, c = l % 3;
            const int r1 = (rr + 1) % 3, r2 = (rr + 2) % 3, c1 = (c + 1) % 3, c2 = (c + 2) % 3;
            Cs[l] = Ms[3 * r1 + c1] * Ms[3 * r2 + c2] - Ms[3 * r1 + c2] * Ms[3 * r2 + c1];
        }
        const double d = Ms[0] * Cs[0] + Ms[1] * Cs[1] + Ms[2] * Cs[2];
        const double inv = 1.0 / d;
        for (int vv = 0; vv < 4; ++vv)
            for (int rr = 0; rr < 3; ++rr)
                g.gl[vv][rr] = vv == 0 ? (-(Cs[3 * rr] * inv) - Cs[3 * rr + 1] * inv) - Cs[3 * rr + 2] * inv
                                       : Cs[3 * rr + vv - 1] * inv;
        g.absdet = fabs(d);
        for (int vv = 0; vv < 4; ++vv)
            for (int rr = 0; rr < 3; ++rr) {
                double sum = 0.;
                for (int i = 0; i < 4; ++i) sum += ls10[i] * ((i == vv ? 3. : -1.) * g.gl[i][rr]);
                for (int k = 0; k < 6; ++k) {
                    const int ea = ev0(k), eb = ev1(k);
                    if (eb == vv) sum += ls10[4 + k] * (4. * g.gl[ea][rr]);
                    if (ea == vv) sum += ls10[4 + k] * (4. * g.gl[eb][rr]);
                }
                g.G[vv][rr] = sum;
            }
        // warp_patch, lane by lane: cut points of the lattice edges, the sub-tets' facets in order
        double lat[10];
        for (int k = 0; k < 10; ++k) lat[cP2OnLat[k]] = ls10[k];
        double cut[25][4];
        for (int k = 0; k < 25; ++k) {
            const int a = cT.edge_a[k], b = cT.edge_b[k];
            const double va = lat[a], vb = lat[b];
            if ((va > 0. && vb < 0.) || (va < 0. && vb > 0.)) cut_point(lat, a, b, cut[k]);
        }
        int nf = 0;
        for (int sub = 0; sub < 8; ++sub) {
            int pat = 0;
            for (int k = 0; k < 4; ++k) {
                const double val = lat[cT.lat_t[sub][k]];
                pat += ((val > 0.) - (val < 0.) + 1) * (k == 0 ? 1 : k == 1 ? 3 : k == 2 ? 9 : 27);
            }
            int nfs = cT.pat_nf[pat];
            if (nfs < 0) {
                set_status(A.status, TF_ERR_ZERO_PATTERN, t);
                nfs = 0;
            }
            for (int f = 0; f < nfs && nf < 16; ++f, ++nf) {
                double w[3][3];
                for (int j = 0; j < 3; ++j) {
                    const int ext = cT.pat_f[pat][f][j];
                    double b[4];
                    if (ext < 4) {
                        const int Lv = cT.lat_t[sub][ext];
                        for (int c = 0; c < 4; ++c) b[c] = cT.lat_v[Lv][c];
                    } else {
                        const int id = cT.ledge[sub][ext - 4];
                        for (int c = 0; c < 4; ++c) b[c] = cut[id][c];
                    }
                    for (int c = 0; c < 4; ++c) Q.fb[nf][j][c] = ff_split(b[c]);
                    for (int rr = 0; rr < 3; ++rr)
                        w[j][rr] = g.X[0][rr] * b[0] + g.X[1][rr] * b[1] + g.X[2][rr] * b[2] + g.X[3][rr] * b[3];
                }
                double u[3], vq[3];
                for (int rr = 0; rr < 3; ++rr) {
                    u[rr] = w[1][rr] - w[0][rr];
                    vq[rr] = w[2][rr] - w[0][rr];
                }
                const double c0 = u[1] * vq[2] - u[2] * vq[1], c1 = u[2] * vq[0] - u[0] * vq[2],
                             c2 = u[0] * vq[1] - u[1] * vq[0];
                Q.fw[nf] = ff_split(sqrt(c0 * c0 + c1 * c1 + c2 * c2) * (cT.pat_bnd[pat] ? 0.5 : 1.0));
            }
        }
        Q.nf = nf;
        // linear level set on the tet: every edge value the mean of its end values, bit for bit
        bool lin = LIN;
        for (int k = 0; LIN && k < 6; ++k) {
            const double mean = __dmul_rn(0.5, __dadd_rn(ls10[ev0(k)], ls10[ev1(k)]));
            lin = lin && __double_as_longlong(mean) == __double_as_longlong(ls10[4 + k]);
        }
        Q.lin = lin;
        if (lin) {
            const double bc[4] = {0.25, 0.25, 0.25, 0.25};
            double n[3];
            unit_normal(g, bc, n);
            for (int vv = 0; vv < 4; ++vv) {
                const double ng = n[0] * g.gl[vv][0] + n[1] * g.gl[vv][1] + n[2] * g.gl[vv][2];
                for (int c = 0; c < 3; ++c) Q.lin_sg[vv][c] = g.gl[vv][c] - ng * n[c];
            }
            for (int k = 0; k < 10; ++k) {
                int i, j;
                sym_entry(4, k, i, j);
                Q.lin_G[k] = Q.lin_sg[j][0] * Q.lin_sg[i][0] + Q.lin_sg[j][1] * Q.lin_sg[i][1] +
                             Q.lin_sg[j][2] * Q.lin_sg[i][2];
            }
            for (int i = 0; i < 4; ++i) Q.lin_dn[i] = n[0] * g.gl[i][0] + n[1] * g.gl[i][1] + n[2] * g.gl[i][2];
        }
        Q.absdet = g.absdet;
        Q.absdet_ff = ff_split(g.absdet);
        for (int vv = 0; vv < 4; ++vv)
            for (int c = 0; c < 3; ++c) {
                Q.gl[vv][c] = ff_split(g.gl[vv][c]);
                Q.G[vv][c] = ff_split(g.G[vv][c]);
                Q.X[vv][c] = ff_split(g.X[vv][c]);
            }
    }
}

// Sort key of a tet for k_prep_tets: the signs (-, 0, +) of its 10 lattice
// values in base 3.  They fix every branch of the prep (which lattice edges
// are cut, each sub-tet's pattern and facets).  Signs from the bits: -0 and
// +0 are zero, NaN counts by its sign bit (the key only orders the threads).
constexpr int kPrepKeyBits = 16;  // 3^10 = 59,049 < 2^16
__global__ void k_prep_key(AsmArgs A, uint32_t* __restrict__ key, int32_t* __restrict__ idx) {
    const int64_t n = A.c1 - A.c0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t v[4], e[6];
        mesh_tet(A.M, A.active[A.c0 + i], v, e);
        uint32_t k = 0;
        for (int j = 0; j < 10; ++j) {
            const unsigned long long b =
                (unsigned long long)__double_as_longlong(j < 4 ? A.lsv[v[j]] : A.lse[e[j - 4]]);
            const uint32_t sg = (b << 1) == 0ull ? 1u : (b >> 63) ? 0u : 2u;
            k = 3u * k + sg;
        }
        key[i] = k;
        idx[i] = (int32_t)i;
    }
}

__global__ void __launch_bounds__(32 * kAsmWarps) k_assemble_p2_pair(AsmArgs A) {
    constexpr int NL = 10, NSYM = 55, EPL = 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    AsmPairSmem& S = reinterpret_cast<AsmPairSmem*>(smem_raw)[wib];
    const bool wantM = A.forms & (1u << TF_FORM_M), wantA = A.forms & (1u << TF_FORM_A);
    const bool wantC = A.forms & (1u << TF_FORM_CN);
    const bool wantF = A.rhs.kind != TF_RHS_NONE;
    const int64_t nwarps = (int64_t)gridDim.x * kAsmWarps;

    const TetPrep* const prep = reinterpret_cast<const TetPrep*>(A.prep);
    for (int64_t r = A.c0 + (int64_t)blockIdx.x * kAsmWarps + wib; r < A.c1; r += nwarps) {
        // the tet's record (k_prep_tets): gl, G, X, |det| and the facets as pairs
        const TetPrep& Q = prep[r - A.c0];
        const int nf = Q.nf;
        for (int k = lane; k < 37; k += 32) {
            const int m = k / 12, v3 = (k % 12) / 3, c = k % 3;
            if (k == 36)
                S.absdet = Q.absdet_ff;
            else
                (m == 0 ? S.gl : m == 1 ? S.G : S.X)[v3][c] = (m == 0 ? Q.gl : m == 1 ? Q.G : Q.X)[v3][c];
        }
        for (int k = lane; k < 13 * nf; k += 32) {
            const int f = k / 13, j = k % 13;
            if (j == 12)
                S.fw[f] = Q.fw[f];
            else
                S.fb[f][j >> 2][j & 3] = Q.fb[f][j >> 2][j & 3];
        }
        __syncwarp();
        AsmPairPts& P = S.u.p;

        ffacc accM[EPL], accA[EPL], accF;
        const int npts = 7 * nf;
        for (int base = 0; base < npts; base += 32) {
            const int p = base + lane;
            if (p < npts) {
                const int f = p / 7, q = p - 7 * (p / 7);
                ff b[4];
                for (int c = 0; c < 4; ++c)
                    b[c] = ff_fma(S.fb[f][2][c], cTF.q2_node[q][2],
                                  ff_fma(S.fb[f][1][c], cTF.q2_node[q][1], ff_mul(S.fb[f][0][c], cTF.q2_node[q][0])));
                const ff sw = ff_sqrt(ff_mul(S.fw[f], cTF.q2_w[q]));
                ff n[3];
                ff_normal(S, b, n);
                // The basis loops are kept rolled (their operands in L1-resident local
                // memory): unrolled, the per-point pair code overflows the instruction cache.
                ff pg[4][3], q4[4];
#pragma unroll 1
                for (int k = 0; k < 4; ++k) {
                    const ff ng = ff_dot3(n, S.gl[k]);
                    for (int c = 0; c < 3; ++c) pg[k][c] = ff_mul(sw, ff_sub(S.gl[k][c], ff_mul(ng, n[c])));
                    q4[k] = ff_scale(b[k], 4.f);
                }
#pragma unroll 1
                for (int i = 0; i < 10; ++i) {
                    // vertex i: phi = b_i (2 b_i - 1), grad = (4 b_i - 1) grad(b_i);
                    // edge (a, c): phi = 4 b_a b_c, grad = 4 b_c grad(b_a) + 4 b_a grad(b_c)
                    const int a = i < 4 ? i : ev0(i - 4), c2 = i < 4 ? i : ev1(i - 4);
                    const ff ph = i < 4 ? ff_mul(b[a], ff_add_f(ff_scale(b[a], 2.f), -1.f)) : ff_mul(q4[a], b[c2]);
                    P.phi[lane][i] = ff_mul(sw, ph);
                    const ff fa = i < 4 ? ff_add_f(q4[a], -1.f) : q4[c2];
                    for (int c = 0; c < 3; ++c) {
                        const ff t = ff_mul(fa, pg[a][c]);
                        P.sg[lane][3 * i + c] = i < 4 ? t : ff_fma(q4[a], pg[c2][c], t);
                    }
                }
                if (wantF) {
                    ff x[3];
                    for (int c = 0; c < 3; ++c)
                        x[c] = ff_fma(b[3], S.X[3][c],
                                      ff_fma(b[2], S.X[2][c], ff_fma(b[1], S.X[1][c], ff_mul(b[0], S.X[0][c]))));
                    S.fx[lane] = ff_mul(sw, ff_rhs(A.rhs, x));
                }
            }
            __syncwarp();
            const int cnt = min(32, npts - base);
            // entries k0 = lane and k1 = lane + 32 in one pass (lanes past the 55th entry repeat
            // the last one and do not store it)
            const int k1 = min(lane + 32, NSYM - 1);
            const int i0 = cT.sym_i[lane], j0 = cT.sym_j[lane], i1 = cT.sym_i[k1], j1 = cT.sym_j[k1];
            for (int pp = 0; pp < cnt; ++pp) {
                if (wantM) {
                    accM[0].add_prod(P.phi[pp][j0], P.phi[pp][i0]);
                    accM[1].add_prod(P.phi[pp][j1], P.phi[pp][i1]);
                }
                if (wantA)
                    for (int c = 0; c < 3; ++c) {
                        accA[0].add_prod(P.sg[pp][3 * j0 + c], P.sg[pp][3 * i0 + c]);
                        accA[1].add_prod(P.sg[pp][3 * j1 + c], P.sg[pp][3 * i1 + c]);
                    }
            }
            if (wantF && lane < 30) {  // 10 rows x 3 point groups (combined after the last chunk)
                const int i = lane % 10;
                for (int pp = lane / 10; pp < cnt; pp += 3) accF.add_prod(S.fx[pp], P.phi[pp][i]);
            }
            __syncwarp();
        }
        ff Fv = ff_of(0.f);
        if (wantF) {  // point groups (g0 + g1) + g2
            const ff f0 = accF.value();
            const ff f1{__shfl_down_sync(0xffffffffu, f0.h, 10), __shfl_down_sync(0xffffffffu, f0.l, 10)};
            const ff f2{__shfl_down_sync(0xffffffffu, f0.h, 20), __shfl_down_sync(0xffffffffu, f0.l, 20)};
            Fv = ff_add(ff_add(f0, f1), f2);
        }
        ffacc accC[EPL];
        if (wantC) {
            // normal-gradient volume stabilisation on the 15-point Quad5 rule
            if (lane < 15) {
                ff b[4];
                for (int c = 0; c < 4; ++c) b[c] = cTF.q3_node[lane][c];
                ff n[3];
                ff_normal(S, b, n);
                ff ng[4];
                for (int k = 0; k < 4; ++k) ng[k] = ff_mul(cTF.q3_sw[lane], ff_dot3(n, S.gl[k]));
                for (int i = 0; i < 4; ++i) P.phi[lane][i] = ff_mul(ff_add_f(ff_scale(b[i], 4.f), -1.f), ng[i]);
                for (int k = 0; k < 6; ++k) {
                    const int a = ev0(k), c2 = ev1(k);
                    P.phi[lane][4 + k] = ff_scale(ff_fma(b[c2], ng[a], ff_mul(b[a], ng[c2])), 4.f);
                }
            }
            __syncwarp();
            const int k1 = min(lane + 32, NSYM - 1);
            const int i0 = cT.sym_i[lane], j0 = cT.sym_j[lane], i1 = cT.sym_i[k1], j1 = cT.sym_j[k1];
            for (int pp = 0; pp < 15; ++pp) {
                accC[0].add_prod(P.phi[pp][j0], P.phi[pp][i0]);
                accC[1].add_prod(P.phi[pp][j1], P.phi[pp][i1]);
            }
            __syncwarp();
        }
        for (int qq = 0; qq < EPL; ++qq) {
            const int k = lane + 32 * qq;
            if (k >= NSYM) break;
            if (wantM) A.elem[((int64_t)TF_FORM_M * A.n_active + r) * NSYM + k] = ff_to_double(accM[qq].value());
            if (wantA) A.elem[((int64_t)TF_FORM_A * A.n_active + r) * NSYM + k] = ff_to_double(accA[qq].value());
            if (wantC)
                A.elem[((int64_t)TF_FORM_CN * A.n_active + r) * NSYM + k] =
                    ff_to_double(ff_mul(accC[qq].value(), S.absdet));
        }
        if (wantF && lane < NL) A.elem_rhs[r * NL + lane] = ff_to_double(Fv);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// P1 forms M, A, C_n and the load vector in pair arithmetic (k_assemble_p1_pair).
// The structure of k_assemble<4>: on a tet whose level set is linear (every
// edge value the mean of its end values, bit for bit) the normal and the hat
// functions' surface gradients are constant, A = (sum_p w_p) sg_i.sg_j and
// C_n = |det| (sum_q w_q) dn_i dn_j from FP64 per-tet constants; otherwise the
// normal, the projected gradients and the 15-point volume rule run per point.
// Per point (node, weight and its square root, normal, gradients, load
// function) and every sum over points run in pair arithmetic; the point
// groups of the sums are those of k_assemble<4> (entries on 3 groups of
// 10 lanes, the load vector on 8 groups of 4).
// ---------------------------------------------------------------------------
struct AsmPair1Pts {
    ff phi[32][5];  // sqrt(w) b_i; n . grad(b_i) sqrt(w_q) for the volume rule (odd pitch: no bank conflicts)
    ff sg[32][13];  // [3 i + c]: sqrt(w) (I - n n^T) grad(b_i)
};
struct AsmPair1Smem {
    AsmPair1Pts p;
    ff gl[4][3], G[4][3], X[4][3];
    ff fb[16][3][4], fw[16];
    ff wt[32], fx[32];  // w_p; sqrt(w) f(x_p)
    double lin_sg[4][3], lin_G[10], lin_dn[4];
};

__device__ __forceinline__ ff ff_shfl_down(ff a, int d) {
    return ff{__shfl_down_sync(0xffffffffu, a.h, d), __shfl_down_sync(0xffffffffu, a.l, d)};
}

__device__ __noinline__ void ff_normal1(const ff (*G)[3], const ff b[4], ff n[3]) {
    ff v[3];
    for (int r = 0; r < 3; ++r) {
        v[r] = ff_mul(b[0], G[0][r]);
        for (int k = 1; k < 4; ++k) v[r] = ff_fma(b[k], G[k][r], v[r]);
    }
    const ff nn = ff_fma(v[2], v[2], ff_fma(v[1], v[1], ff_mul(v[0], v[0])));
    const ff inv = ff_rsqrt(nn);
    for (int r = 0; r < 3; ++r) n[r] = ff_mul(v[r], inv);
}

__global__ void __launch_bounds__(32 * kAsmWarps) k_assemble_p1_pair(AsmArgs A) {
    constexpr int NL = 4, NSYM = 10;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    AsmPair1Smem& S = reinterpret_cast<AsmPair1Smem*>(smem_raw)[wib];
    const bool wantM = A.forms & (1u << TF_FORM_M), wantA = A.forms & (1u << TF_FORM_A);
    const bool wantC = A.forms & (1u << TF_FORM_CN);
    const bool wantF = A.rhs.kind != TF_RHS_NONE;
    const int64_t nwarps = (int64_t)gridDim.x * kAsmWarps;
    double s3 = 0.;  // the 15-point rule's weight sum (linear level set: n . grad(phi_i) is constant)
    for (int pp = 0; pp < 15; ++pp) s3 += cT.q3_w[pp];

    const TetPrep* const prep = reinterpret_cast<const TetPrep*>(A.prep);
    for (int64_t r = A.c0 + (int64_t)blockIdx.x * kAsmWarps + wib; r < A.c1; r += nwarps) {
        // the tet's record (k_prep_tets) into shared memory
        const TetPrep& Q = prep[r - A.c0];
        const int nf = Q.nf;
        const bool lin = Q.lin != 0;
        const double absdet = Q.absdet;
        for (int k = lane; k < 36; k += 32) {
            const int m = k / 12, v3 = (k % 12) / 3, c = k % 3;
            (m == 0 ? S.gl : m == 1 ? S.G : S.X)[v3][c] = (m == 0 ? Q.gl : m == 1 ? Q.G : Q.X)[v3][c];
        }
        for (int k = lane; k < 13 * nf; k += 32) {
            const int f = k / 13, j = k % 13;
            if (j == 12)
                S.fw[f] = Q.fw[f];
            else
                S.fb[f][j >> 2][j & 3] = Q.fb[f][j >> 2][j & 3];
        }
        if (lin)
            for (int k = lane; k < 26; k += 32) {
                if (k < 12)
                    S.lin_sg[k / 3][k % 3] = Q.lin_sg[k / 3][k % 3];
                else if (k < 22)
                    S.lin_G[k - 12] = Q.lin_G[k - 12];
                else
                    S.lin_dn[k - 22] = Q.lin_dn[k - 22];
            }
        __syncwarp();
        AsmPair1Pts& P = S.p;

        ffacc accM, accA, accF;
        const int grp = lane / 10, k10 = lane % 10;
        int ei, ej;
        sym_entry(4, k10, ei, ej);
        const int npts = 7 * nf;
        for (int base = 0; base < npts; base += 32) {
            const int p = base + lane;
            if (p < npts) {
                const int f = p / 7, q = p - 7 * (p / 7);
                ff b[4];
                for (int c = 0; c < 4; ++c)
                    b[c] = ff_fma(S.fb[f][2][c], cTF.q2_node[q][2],
                                  ff_fma(S.fb[f][1][c], cTF.q2_node[q][1], ff_mul(S.fb[f][0][c], cTF.q2_node[q][0])));
                const ff w = ff_mul(S.fw[f], cTF.q2_w[q]);
                const ff sw = ff_sqrt(w);
                S.wt[lane] = w;
                for (int i = 0; i < 4; ++i) P.phi[lane][i] = ff_mul(sw, b[i]);
                if (!lin) {
                    ff n[3];
                    ff_normal1(S.G, b, n);
#pragma unroll 1
                    for (int k = 0; k < 4; ++k) {
                        const ff ng = ff_dot3(n, S.gl[k]);
                        for (int c = 0; c < 3; ++c) P.sg[lane][3 * k + c] = ff_mul(sw, ff_sub(S.gl[k][c], ff_mul(ng, n[c])));
                    }
                }
                if (wantF) {
                    ff x[3];
                    for (int c = 0; c < 3; ++c)
                        x[c] = ff_fma(b[3], S.X[3][c],
                                      ff_fma(b[2], S.X[2][c], ff_fma(b[1], S.X[1][c], ff_mul(b[0], S.X[0][c]))));
                    S.fx[lane] = ff_mul(sw, ff_rhs(A.rhs, x));
                }
            }
            __syncwarp();
            const int cnt = min(32, npts - base);
            if (grp < 3) {
                for (int pp = grp; pp < cnt; pp += 3) {
                    if (wantM) accM.add_prod(P.phi[pp][ej], P.phi[pp][ei]);
                    if (wantA) {
                        if (lin) {
                            accA.add(S.wt[pp]);
                        } else {
                            accA.add_prod(P.sg[pp][3 * ej], P.sg[pp][3 * ei]);
                            accA.add_prod(P.sg[pp][3 * ej + 1], P.sg[pp][3 * ei + 1]);
                            accA.add_prod(P.sg[pp][3 * ej + 2], P.sg[pp][3 * ei + 2]);
                        }
                    }
                }
            }
            if (wantF)
                for (int pp = lane >> 2; pp < cnt; pp += 8) accF.add_prod(S.fx[pp], P.phi[pp][lane & 3]);
            __syncwarp();
        }
        // point groups: entries (g0 + g1) + g2, the load vector a tree over 8 groups
        ff vM = accM.value(), vA = accA.value(), vF = accF.value();
        vM = ff_add(ff_add(vM, ff_shfl_down(vM, 10)), ff_shfl_down(vM, 20));
        vA = ff_add(ff_add(vA, ff_shfl_down(vA, 10)), ff_shfl_down(vA, 20));
        vF = ff_add(vF, ff_shfl_down(vF, 16));
        vF = ff_add(vF, ff_shfl_down(vF, 8));
        vF = ff_add(vF, ff_shfl_down(vF, 4));
        double outC = 0.;
        if (wantC) {
            if (lin) {
                outC = (s3 * (S.lin_dn[ej] * S.lin_dn[ei])) * absdet;
            } else {
                __syncwarp();
                if (lane < 15) {
                    ff b[4];
                    for (int c = 0; c < 4; ++c) b[c] = cTF.q3_node[lane][c];
                    ff n[3];
                    ff_normal1(S.G, b, n);
                    for (int k = 0; k < 4; ++k) P.phi[lane][k] = ff_mul(cTF.q3_sw[lane], ff_dot3(n, S.gl[k]));
                }
                __syncwarp();
                ffacc accC;
                if (grp < 3)
                    for (int pp = grp; pp < 15; pp += 3) accC.add_prod(P.phi[pp][ej], P.phi[pp][ei]);
                ff vC = accC.value();
                vC = ff_add(ff_add(vC, ff_shfl_down(vC, 10)), ff_shfl_down(vC, 20));
                outC = ff_to_double(vC) * absdet;
            }
        }
        if (lane < NSYM) {
            if (wantM) A.elem[((int64_t)TF_FORM_M * A.n_active + r) * NSYM + lane] = ff_to_double(vM);
            if (wantA) {
                const double a = ff_to_double(vA);
                A.elem[((int64_t)TF_FORM_A * A.n_active + r) * NSYM + lane] = lin ? a * S.lin_G[lane] : a;
            }
            if (wantC) A.elem[((int64_t)TF_FORM_CN * A.n_active + r) * NSYM + lane] = outC;
        }
        if (wantF && lane < NL) A.elem_rhs[r * NL + lane] = ff_to_double(vF);
        __syncwarp();
    }
}
