// Tree tensor network (TTN) ground-state sweep: the TenNetLib TTN path (StateEnvsTTN,
// LinkTensorsTTN, moveisometry_to_next!, update_position!, fullsweep!) restated for one GPU,
// behind the tn_ttn_* C ABI of include/tennet.h.
//
// Environments created together form a group: one device arena holds the node tensors and
// link tensors of all of them, and every operation of a sweep runs on the whole group in
// lockstep, so each contraction stage of all instances is one grouped GEMM launch and each
// Krylov vector operation one batched kernel.
//
// Link tensors.  For a Hamiltonian given as product terms, the tensors on a link (u, v)
// oriented toward v describe u's side: one "local" matrix (the sum of all terms that lie
// entirely on u's side, contracted with u's side of the state) and one matrix per term
// that has sites on both sides (its operators on u's side, contracted).  This is
// move_linktensors_to_next! (TenNetLib src/ttn/linktensors.jl:63-118), whose order-<=2
// results are the local matrix and whose order-3 results are the per-term ones.
//
// H_eff at node v is the sum over term groups of mode products: a local matrix acts on one
// leg, a term with factors on k of v's legs acts with one matrix on each of them (k - 1
// chained stages into temporaries, the last factor in the final round of its leg).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <numeric>
#include <set>
#include <string>

#include "engine.h"
#include "ttn_internal.h"

using namespace tn;

// -------------------------------------------------------------------------------------
// tree
// -------------------------------------------------------------------------------------
int TtnTree::leg_nbr(int v, int u) const {
    for (size_t i = 0; i < nbr[v].size(); ++i)
        if (nbr[v][i] == u) return int(sites[v].size() + i);
    return -1;
}
int TtnTree::leg_site(int v, int n) const {
    for (size_t i = 0; i < sites[v].size(); ++i)
        if (sites[v][i] == n) return int(i);
    return -1;
}
int TtnTree::edge(int a, int b) const {
    auto it = eidx.find({std::min(a, b), std::max(a, b)});
    return it == eidx.end() ? -1 : it->second;
}
std::vector<int> TtnTree::path(int a, int b) const {
    std::vector<int> par(nn, -2);
    std::deque<int> q{a};
    par[a] = -1;
    while (!q.empty()) {
        const int x = q.front();
        q.pop_front();
        if (x == b) break;
        for (int y : nbr[x])
            if (par[y] == -2) {
                par[y] = x;
                q.push_back(y);
            }
    }
    TN_REQUIRE(par[b] != -2, "TTN: nodes are not connected");
    std::vector<int> out{b};
    while (out.back() != a) out.push_back(par[out.back()]);
    std::reverse(out.begin(), out.end());
    return out;
}
std::vector<char> TtnTree::side(int v, int u) const {
    std::vector<char> in(N, 0), seen(nn, 0);
    std::vector<int> st{v};
    seen[v] = seen[u] = 1;
    while (!st.empty()) {
        const int x = st.back();
        st.pop_back();
        for (int s : sites[x]) in[s] = 1;
        for (int y : nbr[x])
            if (!seen[y]) {
                seen[y] = 1;
                st.push_back(y);
            }
    }
    return in;
}

namespace {

int64_t prod(const std::vector<int>& d, int lo, int hi) {
    int64_t p = 1;
    for (int i = lo; i < hi; ++i) p *= d[i];
    return p;
}
int64_t vol(const std::vector<int>& d) { return prod(d, 0, int(d.size())); }

TtnTree make_tree(int N, int d, int nn, int ne, const int32_t* edges, const int32_t* site_node) {
    TN_REQUIRE(N >= 1 && d >= 1 && nn >= 1, "TTN: empty tree");
    TN_REQUIRE(ne == nn - 1, "TTN: a tree of n nodes has n - 1 edges");
    TtnTree t;
    t.N = N;
    t.d = d;
    t.nn = nn;
    t.nbr.assign(nn, {});
    t.sites.assign(nn, {});
    t.site_node.assign(site_node, site_node + N);
    for (int i = 0; i < N; ++i) {
        TN_REQUIRE(site_node[i] >= 0 && site_node[i] < nn, "TTN: site on a missing node");
        t.sites[site_node[i]].push_back(i);
    }
    for (int e = 0; e < ne; ++e) {
        const int a = edges[2 * e], b = edges[2 * e + 1];
        TN_REQUIRE(a >= 0 && a < nn && b >= 0 && b < nn && a != b, "TTN: bad edge");
        const auto key = std::make_pair(std::min(a, b), std::max(a, b));
        TN_REQUIRE(!t.eidx.count(key), "TTN: repeated edge");
        t.eidx[key] = int(t.edges.size());
        t.edges.push_back(key);
        t.nbr[a].push_back(b);
        t.nbr[b].push_back(a);
    }
    for (auto& v : t.nbr) std::sort(v.begin(), v.end());
    // connected (n - 1 edges + connected = tree)
    std::vector<char> seen(nn, 0);
    std::vector<int> st{0};
    seen[0] = 1;
    int cnt = 1;
    while (!st.empty()) {
        const int x = st.back();
        st.pop_back();
        for (int y : t.nbr[x])
            if (!seen[y]) {
                seen[y] = 1;
                ++cnt;
                st.push_back(y);
            }
    }
    TN_REQUIRE(cnt == nn, "TTN: the graph is not connected (or has a loop)");
    for (int v = 0; v < nn; ++v) TN_REQUIRE(t.nlegs(v) >= 1, "TTN: node without legs");
    return t;
}

// nodes ordered farthest-first from c (ties by node number): nodes_from_bfs(...; reverse)
std::vector<int> bfs_reverse(const TtnTree& t, int c) {
    std::vector<int> dist(t.nn, -1);
    std::deque<int> q{c};
    dist[c] = 0;
    while (!q.empty()) {
        const int x = q.front();
        q.pop_front();
        for (int y : t.nbr[x])
            if (dist[y] < 0) {
                dist[y] = dist[x] + 1;
                q.push_back(y);
            }
    }
    std::vector<int> order(t.nn);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return dist[a] > dist[b]; });
    return order;
}

template <class F>
int guarded(F&& f) {
    try {
        f();
        return TN_OK;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return TN_E_NOMEM;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return TN_E_INVALID;
    }
}

}  // namespace

// -------------------------------------------------------------------------------------
// handles
// -------------------------------------------------------------------------------------
struct tn_ttn {
    tn_ctx* ctx = nullptr;
    TtnTree tree;
    std::vector<std::vector<int>> dims;  // per node, per leg
    std::vector<DevBuf> node;
    int center = -1;
};

struct tn_ttn_model {
    int N = 0, d = 0;
    struct Term {
        std::vector<int> sites;                 // ascending
        std::vector<std::vector<double>> ops;   // d*d each, coefficient on the first
    };
    std::vector<Term> terms;
};

namespace {

// one factor of a term group: the matrix at arena offset moff acting on leg `leg`
struct Piece {
    int leg;
    int64_t moff;
};
struct TGroup {
    int term;  // -1: a local matrix
    std::vector<Piece> pcs;
};

// a grouped GEMM plan with its split-precision form (packs in group scratch)
struct TPlan {
    GemmPlan g;
    std::unique_ptr<SplitPlan> sp;
    bool finalized = false;
};

struct ProductPlan {    // H_eff x at one node
    std::vector<TPlan> stages;  // chained factors of groups with several (stage j: factor j)
    std::vector<TPlan> rounds;
    double flops = 0;
};
struct MovePlan {       // link tensors of edge (v -> u)
    std::vector<TPlan> stages;
    std::vector<TPlan> rounds;
    TPlan tg;
    CombPlan comb;
    double flops = 0;
};
struct QrPlan {         // isometry move v -> u: blocked-QR GEMMs and the R mode product
    std::vector<TPlan> w, w2, upd;       // per panel (factorisation)
    std::vector<CombPlan> wc;
    // Q formation with the whole block reflector: G = V^T V (k split, then combined),
    // W = (-T) V_top^T, Q = [I; 0] + V W
    TPlan gram, qw, qfin;
    CombPlan gramc;
    TPlan rmode;
    int npanel = 0;
};

}  // namespace

// One state M of an excited-state projector (LinkProjTTN, TenNetLib src/ttn/linkproj.jl:15-224):
// M's node tensors and, per tree link, the overlap matrix of psi and M on one side of it
// (psi's link index first, leading dimension psi's link dimension), oriented toward the
// orthogonality centre like the link tensors.
struct TtnProj {
    std::vector<std::vector<int>> mdims;  // M's node dimensions (legs ordered as psi's)
    std::vector<int64_t> moff;            // node offsets in mbuf
    DevBuf mbuf;
    std::vector<int64_t> eoff;            // per edge: overlap matrix offset in ebuf
    std::vector<int> efrom;               // node whose side the overlap describes (-1: none yet)
    DevBuf ebuf;
};

struct TtnGroup;

struct tn_ttn_env {
    std::shared_ptr<TtnGroup> grp;
    int idx = 0;
    tn_ctx* ctx = nullptr;
    TtnTree tree;
    tn_ttn_model model;
    std::vector<std::vector<int>> dims;
    int center = -1;
    // arena layout (slot S_L)
    std::vector<int64_t> node_off;
    struct SiteStore {
        int64_t local = -1;
        std::map<int, int64_t> open;  // term -> offset
    };
    std::vector<SiteStore> sstore;
    struct EdgeStore {
        int64_t off = 0;
        int cap_dim = 0;
        std::vector<int> cross;       // terms with sites on both sides, ascending
        int from = -1;                // node whose side the stored tensors describe
        bool local[2] = {false, false};  // local exists when from == edge.first / .second
    };
    std::vector<EdgeStore> estore;
    int64_t arena_size = 0;
    int64_t S = 0;                    // largest node tensor (elements)
    int ntmp = 0;                     // temporaries of one product / link move
    int ncross_max = 0;
    int dmax = 0;                     // largest link dimension
    // work layout (slot S_R), relative to this instance's work base
    int64_t wbase = 0;
    int64_t w_x = 0, w_y = 0, w_kry = 0, w_tmp = 0, w_part = 0, w_qa = 0, w_qv = 0, w_r = 0,
            w_rt = 0, w_tt = 0, w_tau = 0, w_small = 0, w_wp = 0, w_w = 0, w_w2 = 0, w_hpart = 0,
            w_coef = 0, w_g = 0, w_tall = 0, w_wq = 0, w_end = 0;
    int kry_vecs = 0;
    int nchunk_t = 1;                 // k chunks of the link-tensor contractions
    int nchunk_q = 1;                 // k chunks of the QR panel products
    // slot capacities (elements per node slot, set by the arena layout; link dimensions per
    // edge slot: link_cap, or the creation sizes when empty); grow_group raises them when
    // subspace expansion needs room
    std::vector<int64_t> node_cap;
    std::vector<int> link_cap;
    int64_t expand_events = 0;        // subspace expansions so far (the padding stream's counter)
    // excited-state projectors (none when empty): H_eff x + proj_weight sum_k m_k (m_k . x)
    std::vector<TtnProj> proj;
    double proj_weight = 0;
    DevBuf proj_t1, proj_t2, proj_m, proj_c, proj_part;
    int64_t proj_tn = 0;              // elements of one temporary
    // statistics of the last solve
    double energy = 0;
    int matvecs = 0, converged = 0;
};

struct TtnGroup {
    tn_ctx* ctx = nullptr;
    std::vector<tn_ttn_env*> envs;  // members in creation order (null once destroyed)
    int alive = 0;
    DevBuf arena, work, packs, tickets, scal, bpart, bars;
    DevBuf pads, d_cat;  // subspace-expansion padding and its direct-sum descriptors
    DevBuf d_gs, d_sc, d_lin, d_perm, d_qr, d_hh;  // descriptor tables of the batched kernels
    int work_kd = 0;
    std::map<int, std::unique_ptr<ProductPlan>> pcache;
    std::map<std::pair<int, int>, std::unique_ptr<MovePlan>> mcache;
    std::map<std::pair<int, int>, std::unique_ptr<QrPlan>> qcache;
    int dims_version = 0, cache_version = -1;
    double acc_ms[T_NCAT] = {};
    double heff_flops = 0, gemm_flops = 0, krylov_bytes = 0;
    int64_t gemm_launches = 0, matvecs = 0;
};

namespace {

constexpr int SCAL_PER = 160;   // per-instance scalar area (doubles) of the Krylov kernels
constexpr int64_t SMALL_QR = 16384;  // m * n above this: blocked QR (one CTA is FP64-bound)

Bases group_bases(TtnGroup& G) {
    Bases b{};
    b.p[S_L] = G.arena.d();
    b.p[S_R] = G.work.d();
    return b;
}
double* wptr(TtnGroup& G, const tn_ttn_env* e, int64_t off) { return G.work.d() + e->wbase + off; }
double* aptr(TtnGroup& G, int64_t off) { return G.arena.d() + off; }

// ---- grouped GEMM execution ---------------------------------------------------------
void tplan_run(TtnGroup& G, TPlan& p, int slices, int timecat) {
    if (p.g.tasks.empty()) return;
    tn_ctx* ctx = G.ctx;
    cudaStream_t st = ctx->stream;
    if (!p.finalized) {
        p.g.finalize(st);
        p.finalized = true;
    }
    const Bases bs = group_bases(G);
    const int e0 = ctx->timer.mark();
    if (slices == 0) {
        launch_gemm_f64(p.g, bs, st);
    } else {
        if (!p.sp || p.sp->slices != slices) p.sp = make_split_plan(p.g, slices, st, false);
        SplitPlan& sp = *p.sp;
        const size_t need = size_t(sp.abytes + sp.bbytes) + size_t(sp.ea_n + sp.eb_n) * 4 + 4096;
        if (G.packs.bytes < need) G.packs.alloc(need + need / 4, st);
        uint8_t* base = G.packs.as<uint8_t>();
        sp.ap = base;
        sp.bp = base + ((sp.abytes + 1023) / 1024) * 1024;
        uint8_t* e = sp.bp + ((sp.bbytes + 1023) / 1024) * 1024;
        sp.eap = reinterpret_cast<int*>(e);
        sp.ebp = sp.eap + ((sp.ea_n + 63) / 64) * 64;
        run_split_plan(ctx, sp, bs);
    }
    const int e1 = ctx->timer.mark();
    if (timecat == T_HEFF) {
        ctx->timer.add(T_GEMM, e0, e1);
        G.gemm_flops += p.g.flops;
        G.gemm_launches += 1;
    }
}

void comb_run(TtnGroup& G, CombPlan& c) {
    if (c.outs.empty()) return;
    if (c.tiles.empty()) c.finalize(G.ctx->stream);
    launch_combine(c, group_bases(G), G.ctx->stream);
}

int prod_slices(const TtnGroup& G) { return G.ctx->prec == TN_PREC_SPLIT ? G.ctx->slices : 0; }
int qr_slices(const TtnGroup& G) { return G.ctx->prec == TN_PREC_SPLIT ? 7 : 0; }

// ---- mode products --------------------------------------------------------------------
// Y (dims with leg `leg` of size dout) [+]= sum_p M_p x_leg Z_p, M_p dout x dims[leg] (ld dout)
struct ModeIn {
    int zbuf;
    int64_t zoff;
    int mbuf;
    int64_t moff;
};
void add_mode_tasks(GemmPlan& g, const std::vector<int>& dims, int leg, int dout, int ybuf,
                    int64_t yoff, const std::vector<ModeIn>& ins, int accum) {
    if (ins.empty()) return;
    const int64_t P = prod(dims, 0, leg), Q = prod(dims, leg + 1, int(dims.size()));
    const int D = dims[leg];
    if (P == 1) {
        g.add_task(ybuf, yoff, dout, int(Q), dout, accum);
        for (const auto& x : ins) g.add_seg(x.mbuf, x.moff, dout, 0, x.zbuf, x.zoff, D, 0, D);
    } else if (Q == 1) {
        g.add_task(ybuf, yoff, int(P), dout, int(P), accum);
        for (const auto& x : ins) g.add_seg(x.zbuf, x.zoff, int(P), 0, x.mbuf, x.moff, dout, 1, D);
    } else {
        for (int64_t q = 0; q < Q; ++q) {
            g.add_task(ybuf, yoff + q * P * dout, int(P), dout, int(P), accum);
            for (const auto& x : ins)
                g.add_seg(x.zbuf, x.zoff + q * P * D, int(P), 0, x.mbuf, x.moff, dout, 1, D);
        }
    }
}

// T (D x D, at tbuf/toff) = contraction of phi and Y over every leg but `leg`;
// k is split in chunks written to partial buffers and summed by `comb` when large
void add_env_contraction(GemmPlan& g, CombPlan& comb, const std::vector<int>& dims, int leg,
                         int phibuf, int64_t phioff, int ybuf, int64_t yoff, int tbuf, int64_t toff,
                         int partbuf, int64_t partoff, int nchunk_max) {
    const int64_t P = prod(dims, 0, leg), Q = prod(dims, leg + 1, int(dims.size()));
    const int D = dims[leg];
    // units of the k dimension: rows (Q == 1), columns (P == 1) or q slices (middle leg)
    const int64_t units = Q == 1 ? P : Q;
    const int64_t per_unit = Q == 1 || P == 1 ? 1 : P;
    const int64_t ktot = units * per_unit;
    int nch = 1;
    if (ktot >= 4096 && D >= 16) nch = int(std::min<int64_t>(nchunk_max, ktot / 2048));
    nch = std::max(1, std::min<int>(nch, int(units)));
    const int64_t per = (units + nch - 1) / nch;
    std::vector<int64_t> parts;
    for (int c = 0; c < nch; ++c) {
        const int64_t u0 = c * per, u1 = std::min(units, u0 + per);
        if (u0 >= u1) break;
        int cb = tbuf;
        int64_t co = toff;
        if (nch > 1) {
            cb = partbuf;
            co = partoff + int64_t(c) * D * D;
            parts.push_back(co);
        }
        g.add_task(cb, co, D, D, D, 0);
        if (Q == 1) {        // T = Phi^T Y, rows u0..u1
            g.add_seg(phibuf, phioff + u0, int(P), 1, ybuf, yoff + u0, int(P), 0, int(u1 - u0));
        } else if (P == 1) { // T = Phi Y^T, columns u0..u1
            g.add_seg(phibuf, phioff + u0 * D, D, 0, ybuf, yoff + u0 * D, D, 1, int(u1 - u0));
        } else {             // T = sum_q Phi_q^T Y_q
            for (int64_t q = u0; q < u1; ++q)
                g.add_seg(phibuf, phioff + q * P * D, int(P), 1, ybuf, yoff + q * P * D, int(P), 0,
                          int(P));
        }
    }
    if (parts.size() > 1) {
        CombOut o{};
        o.doff = toff;
        o.dbuf = tbuf;
        o.ldd = D;
        o.rows = D;
        o.cols = D;
        o.t0 = int(comb.terms.size());
        o.nt = int(parts.size());
        for (int64_t po : parts) comb.terms.push_back(CombTerm{po, partbuf, D, 1.0});
        comb.outs.push_back(o);
    }
}

// ---- term groups at a node ------------------------------------------------------------
// groups acting on node v's legs (all legs, or all but the leg toward `skip`)
std::vector<TGroup> collect_groups(const tn_ttn_env* e, int v, int skip) {
    const TtnTree& t = e->tree;
    std::vector<TGroup> out;
    std::map<int, TGroup> byterm;
    for (size_t i = 0; i < t.sites[v].size(); ++i) {
        const auto& ss = e->sstore[t.sites[v][i]];
        if (ss.local >= 0) out.push_back(TGroup{-1, {Piece{int(i), ss.local}}});
        for (const auto& kv : ss.open) {
            auto& g = byterm[kv.first];
            g.term = kv.first;
            g.pcs.push_back(Piece{int(i), kv.second});
        }
    }
    for (size_t j = 0; j < t.nbr[v].size(); ++j) {
        const int u = t.nbr[v][j];
        if (u == skip) continue;
        const int leg = int(t.sites[v].size() + j);
        const int eid = t.edge(v, u);
        const auto& es = e->estore[eid];
        TN_REQUIRE(es.from == u, "TTN internal: link tensors are not oriented toward the node");
        const int D = e->dims[v][leg];
        const bool loc = es.local[t.edges[eid].first == u ? 0 : 1];
        if (loc) out.push_back(TGroup{-1, {Piece{leg, es.off}}});
        for (size_t c = 0; c < es.cross.size(); ++c) {
            auto& g = byterm[es.cross[c]];
            g.term = es.cross[c];
            g.pcs.push_back(Piece{leg, es.off + int64_t(1 + c) * D * D});
        }
    }
    for (auto& kv : byterm) out.push_back(std::move(kv.second));
    return out;
}

// order the factors of a group by leg, so that the last one acts on the largest leg
void order_pieces(TGroup& g) {
    std::stable_sort(g.pcs.begin(), g.pcs.end(),
                     [](const Piece& a, const Piece& b) { return a.leg < b.leg; });
}

// ---- per-instance layout -----------------------------------------------------------------
void build_arena_layout(tn_ttn_env* e, int64_t& cursor) {
    const TtnTree& t = e->tree;
    e->node_off.assign(t.nn, 0);
    e->S = 0;
    e->dmax = 1;
    e->node_cap.resize(size_t(t.nn), 0);
    for (int v = 0; v < t.nn; ++v) {
        e->node_off[v] = cursor;
        const int64_t n = std::max(vol(e->dims[v]), e->node_cap[size_t(v)]);
        e->node_cap[size_t(v)] = n;  // the slot's size: what the node tensor may grow to
        cursor += (n + 31) / 32 * 32;
        e->S = std::max(e->S, n);
        for (int x : e->dims[v]) e->dmax = std::max(e->dmax, x);
    }
    const int dd = t.d * t.d;
    e->sstore.assign(t.N, {});
    for (size_t ti = 0; ti < e->model.terms.size(); ++ti) {
        const auto& tm = e->model.terms[ti];
        for (size_t j = 0; j < tm.sites.size(); ++j) {
            auto& ss = e->sstore[tm.sites[j]];
            if (tm.sites.size() == 1) {
                if (ss.local < 0) {
                    ss.local = cursor;
                    cursor += dd;
                }
            } else {
                ss.open[int(ti)] = cursor;
                cursor += dd;
            }
        }
    }
    e->estore.assign(t.edges.size(), {});
    e->ncross_max = 0;
    for (size_t ei = 0; ei < t.edges.size(); ++ei) {
        auto& es = e->estore[ei];
        const int a = t.edges[ei].first, b = t.edges[ei].second;
        const auto sa = t.side(a, b);  // sites on a's side
        es.cap_dim = e->dims[a][t.leg_nbr(a, b)];
        if (ei < e->link_cap.size()) es.cap_dim = std::max(es.cap_dim, e->link_cap[ei]);
        e->dmax = std::max(e->dmax, es.cap_dim);
        for (size_t ti = 0; ti < e->model.terms.size(); ++ti) {
            int ina = 0;
            for (int s : e->model.terms[ti].sites) ina += sa[s];
            const int tot = int(e->model.terms[ti].sites.size());
            if (ina > 0 && ina < tot) es.cross.push_back(int(ti));
            if (ina == tot) es.local[0] = true;   // a term entirely on a's side
            if (ina == 0) es.local[1] = true;     // entirely on b's side
        }
        e->ncross_max = std::max<int>(e->ncross_max, int(es.cross.size()));
        es.off = cursor;
        cursor += int64_t(1 + es.cross.size()) * es.cap_dim * es.cap_dim;
        cursor = (cursor + 31) / 32 * 32;
    }
    // temporaries of one product or link move: k - 1 per group of k factors, one per open
    // group, one for the local sum
    int ntmp = 1;
    for (int v = 0; v < t.nn; ++v) {
        // product at v: a group of k factors chains k - 1 temporaries
        int n2 = 0, nall = 0;
        std::map<int, int> cnt;
        for (int s : t.sites[v])
            for (const auto& kv : e->sstore[s].open) cnt[kv.first]++;
        for (int u : t.nbr[v])
            for (int term : e->estore[t.edge(v, u)].cross) cnt[term]++;
        for (auto& kv : cnt) {
            nall++;
            if (kv.second >= 2) n2 += kv.second - 1;
        }
        ntmp = std::max(ntmp, n2 + nall + 2);
    }
    e->ntmp = ntmp;
}

void build_work_layout(tn_ttn_env* e, int kd) {
    int64_t c = 0;
    const int64_t S = (e->S + 31) / 32 * 32;
    const int64_t D2 = int64_t(e->dmax) * e->dmax;
    auto take = [&](int64_t n) {
        const int64_t o = c;
        c += (n + 31) / 32 * 32;
        return o;
    };
    e->kry_vecs = 2 * kd + 1;
    e->nchunk_t = 32;
    e->nchunk_q = 128;
    e->w_x = take(S);
    e->w_y = take(S);
    e->w_kry = take(S * e->kry_vecs);
    e->w_tmp = take(S * e->ntmp);
    e->w_part = take(int64_t(e->nchunk_t) * (e->ncross_max + 2) * D2);
    e->w_qa = take(S);
    e->w_qv = take(S + int64_t(HH_B) * HH_B);
    e->w_r = take(D2);
    e->w_rt = take(S);
    e->w_tt = take((e->dmax / HH_B + 2) * int64_t(HH_B) * HH_B);
    e->w_tau = take(e->dmax + 32);
    e->w_small = take(64);
    e->w_wp = take(int64_t(e->nchunk_q) * HH_B * e->dmax);
    e->w_w = take(int64_t(HH_B) * e->dmax);
    e->w_w2 = take(int64_t(HH_B) * e->dmax);
    e->w_hpart = take(int64_t(HH_B) * HH_B * TTN_PARTS);
    e->w_coef = take(int64_t(BK_MAX) * BK_MAX);
    e->w_g = take(D2);
    e->w_tall = take(D2);
    e->w_wq = take(D2);
    e->w_end = c;
}

void ensure_work(TtnGroup& G, int kd) {
    if (G.work_kd >= kd && G.work.p) return;
    int64_t total = 0;
    for (auto* e : G.envs) {
        if (!e) continue;
        build_work_layout(e, std::max(kd, 5));
        e->wbase = total;
        total += e->w_end;
    }
    G.work.alloc(size_t(total) * 8, G.ctx->stream);
    G.work_kd = std::max(kd, 5);
    // plans hold work offsets: rebuild
    G.pcache.clear();
    G.mcache.clear();
    G.qcache.clear();
}

std::vector<tn_ttn_env*> members(TtnGroup& G) {
    std::vector<tn_ttn_env*> m;
    for (auto* e : G.envs)
        if (e) m.push_back(e);
    return m;
}

void check_cache(TtnGroup& G) {
    if (G.cache_version != G.dims_version) {
        G.pcache.clear();
        G.mcache.clear();
        G.qcache.clear();
        G.cache_version = G.dims_version;
    }
}

// ---- plans ------------------------------------------------------------------------------
// evaluation of term groups on a source tensor into targets (sum of closed groups, or one
// per open group); rounds[r] holds the r-th leg bucket of every target (r > 0 accumulates)
struct EvalTarget {
    int64_t off;                 // work offset (relative to the instance base)
    std::vector<TGroup> groups;
};
void add_eval(tn_ttn_env* e, const std::vector<int>& dims, int srcbuf, int64_t srcoff,
              std::vector<EvalTarget>& targets, std::vector<TPlan>& stages,
              std::vector<TPlan>& rounds, int tmp_first, double& flops) {
    const int64_t tmpcur = e->w_tmp + int64_t(tmp_first) * ((e->S + 31) / 32 * 32);
    const int64_t n = vol(dims);
    const int64_t S = (e->S + 31) / 32 * 32;
    int tmp_used = 0;
    for (auto& tg : targets) {
        std::map<int, std::vector<ModeIn>> bucket;  // final leg -> inputs
        for (auto& g : tg.groups) {
            order_pieces(g);
            const size_t k = g.pcs.size();
            int zb = srcbuf;
            int64_t zo = srcoff;
            // factors 0 .. k-2 chained through temporaries (stage j applies factor j of every
            // group), the last one in the final round of its leg
            for (size_t j = 0; j + 1 < k; ++j) {
                const int64_t toff = e->wbase + tmpcur + int64_t(tmp_used++) * S;
                TN_REQUIRE(tmp_first + tmp_used <= e->ntmp, "TTN internal: temporaries exhausted");
                if (stages.size() <= j) stages.emplace_back();
                add_mode_tasks(stages[j].g, dims, g.pcs[j].leg, dims[g.pcs[j].leg], S_R, toff,
                               {ModeIn{zb, zo, S_L, g.pcs[j].moff}}, 0);
                flops += 2.0 * n * dims[g.pcs[j].leg];
                zb = S_R;
                zo = toff;
            }
            bucket[g.pcs[k - 1].leg].push_back(ModeIn{zb, zo, S_L, g.pcs[k - 1].moff});
        }
        int r = 0;
        for (auto& kv : bucket) {
            if (int(rounds.size()) <= r) rounds.emplace_back();
            add_mode_tasks(rounds[r].g, dims, kv.first, dims[kv.first], S_R, e->wbase + tg.off,
                           kv.second, r > 0 ? 1 : 0);
            flops += 2.0 * n * dims[kv.first] * double(kv.second.size());
            ++r;
        }
        if (bucket.empty()) {
            // no term acts here: the target is zero (a combine with no terms writes zeros)
            TN_REQUIRE(false, "TTN internal: empty term group set");
        }
    }
}

ProductPlan& product_plan(TtnGroup& G, int v) {
    check_cache(G);
    auto& slot = G.pcache[v];
    if (slot) return *slot;
    slot = std::make_unique<ProductPlan>();
    ProductPlan& P = *slot;
    for (auto* e : members(G)) {
        std::vector<EvalTarget> tg(1);
        tg[0].off = e->w_y;
        tg[0].groups = collect_groups(e, v, -1);
        TN_REQUIRE(!tg[0].groups.empty(), "TTN: the Hamiltonian has no term at this node");
        add_eval(e, e->dims[v], S_R, e->wbase + e->w_x, tg, P.stages, P.rounds, 0, P.flops);
    }
    return P;
}

MovePlan& move_plan(TtnGroup& G, int v, int u) {
    check_cache(G);
    auto& slot = G.mcache[{v, u}];
    if (slot) return *slot;
    slot = std::make_unique<MovePlan>();
    MovePlan& M = *slot;
    const TtnTree& t = members(G)[0]->tree;
    const int eid = t.edge(v, u);
    const auto side = t.side(v, u);
    for (auto* e : members(G)) {
        const auto& dims = e->dims[v];
        const int lu = t.leg_nbr(v, u);
        const int D = dims[lu];
        const auto& es = e->estore[eid];
        const int64_t S = (e->S + 31) / 32 * 32;
        auto groups = collect_groups(e, v, u);
        std::vector<EvalTarget> tg;
        EvalTarget loc;
        loc.off = e->w_tmp;  // first temporary: the local sum
        std::map<int, int64_t> open_slot;
        int next = 1;
        for (auto& g : groups) {
            bool closed = g.term < 0;
            if (!closed) {
                closed = true;
                for (int s : e->model.terms[g.term].sites) closed = closed && side[s];
            }
            if (closed) {
                loc.groups.push_back(g);
            } else {
                EvalTarget o;
                o.off = e->w_tmp + int64_t(next++) * S;
                o.groups.push_back(g);
                tg.push_back(o);
                auto it = std::find(es.cross.begin(), es.cross.end(), g.term);
                TN_REQUIRE(it != es.cross.end(), "TTN internal: open term not crossing the link");
                open_slot[int(tg.size()) - 1] = es.off + int64_t(1 + (it - es.cross.begin())) * D * D;
            }
        }
        const bool has_loc = !loc.groups.empty();
        const bool expect_loc = es.local[t.edges[eid].first == v ? 0 : 1];
        TN_REQUIRE(has_loc == expect_loc, "TTN internal: local link tensor bookkeeping");
        TN_REQUIRE(int(tg.size()) == int(es.cross.size()),
                   "TTN internal: crossing terms and open groups disagree");
        std::vector<EvalTarget> all;
        if (has_loc) all.push_back(loc);
        for (auto& o : tg) all.push_back(o);
        TN_REQUIRE(e->ntmp >= next, "TTN internal: too few temporaries");
        add_eval(e, dims, S_L, e->node_off[v], all, M.stages, M.rounds, next, M.flops);
        // contractions with the node tensor into the link slots
        int pi = 0;
        auto contract = [&](int64_t yoff, int64_t slot_off) {
            add_env_contraction(M.tg.g, M.comb, dims, lu, S_L, e->node_off[v], S_R, e->wbase + yoff,
                                S_L, slot_off, S_R,
                                e->wbase + e->w_part + int64_t(pi++) * e->nchunk_t * D * D,
                                e->nchunk_t);
            M.flops += 2.0 * vol(dims) * D;
        };
        if (has_loc) contract(loc.off, es.off);
        for (size_t i = 0; i < tg.size(); ++i) contract(tg[i].off, open_slot[int(i)]);
    }
    return M;
}

// ---- batched Krylov helpers -------------------------------------------------------------
template <class T>
void upload_descs(TtnGroup& G, DevBuf& buf, const std::vector<T>& v) {
    buf.alloc(std::max<size_t>(v.size() * sizeof(T), 64), G.ctx->stream);
    TN_CUDA(cudaMemcpyAsync(buf.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice,
                            G.ctx->stream));
}




double* scal_of(TtnGroup& G, int i) { return G.scal.d() + int64_t(i) * SCAL_PER; }
unsigned* hh_ticket(TtnGroup& G, int i) { return G.tickets.as<unsigned>() + G.envs.size() + 1 + i; }

void ensure_scal(TtnGroup& G) {
    const size_t n = G.envs.size();
    if (G.scal.bytes < n * SCAL_PER * 8) G.scal.alloc(n * SCAL_PER * 8, G.ctx->stream);
    if (G.bpart.bytes < n * (BK_MAX + 1) * TTN_PARTS * 8)
        G.bpart.alloc(n * (BK_MAX + 1) * TTN_PARTS * 8, G.ctx->stream);
    if (G.tickets.bytes < (2 * n + 2) * sizeof(unsigned)) {
        G.tickets.alloc((2 * n + 2) * sizeof(unsigned), G.ctx->stream);
        TN_CUDA(cudaMemsetAsync(G.tickets.p, 0, G.tickets.bytes, G.ctx->stream));
    }
}

void gs_launch(TtnGroup& G, const std::vector<BGsDesc>& d, int kmax, double sign, bool dots,
               bool norm) {
    if (d.empty()) return;
    int64_t nmax = 1;
    for (const auto& x : d) nmax = std::max(nmax, x.n);
    upload_descs(G, G.d_gs, d);
    launch_bgs_pass(G.d_gs.as<BGsDesc>(), int(d.size()), std::max(kmax, 1), nmax, sign, dots, norm,
                    G.bpart.d(), G.tickets.as<unsigned>(), G.ctx->stream);
    for (const auto& x : d)
        count_krylov_bytes(int64_t(1 + ((x.hin || dots) ? x.kk : 0) + (x.hin ? 1 : 0)) * x.n * 8);
}
void scale_launch(TtnGroup& G, const std::vector<BScaleDesc>& d) {
    if (d.empty()) return;
    int64_t nmax = 1;
    for (const auto& x : d) nmax = std::max(nmax, x.n);
    upload_descs(G, G.d_sc, d);
    launch_bscale(G.d_sc.as<BScaleDesc>(), int(d.size()), nmax, G.ctx->stream);
    for (const auto& x : d) count_krylov_bytes(int64_t(x.dst2 ? 3 : 2) * x.n * 8);
}
void lin_launch(TtnGroup& G, const std::vector<BLinDesc>& d) {
    if (d.empty()) return;
    int64_t nmax = 1;
    for (const auto& x : d) nmax = std::max(nmax, x.n);
    upload_descs(G, G.d_lin, d);
    launch_blincomb(G.d_lin.as<BLinDesc>(), int(d.size()), nmax, G.ctx->stream);
    for (const auto& x : d) count_krylov_bytes(int64_t(x.kk + 1) * x.n * 8);
}

// x_i /= |x_i| in place for every listed instance (norm into scal[64])
void normalize_batch(TtnGroup& G, const std::vector<tn_ttn_env*>& E,
                     const std::vector<double*>& x, const std::vector<int64_t>& n) {
    ensure_scal(G);
    std::vector<BGsDesc> gs(E.size());
    std::vector<BScaleDesc> sc(E.size());
    for (size_t i = 0; i < E.size(); ++i) {
        gs[i] = BGsDesc{};
        gs[i].w = x[i];
        gs[i].out = scal_of(G, E[i]->idx) + 64;
        gs[i].n = n[i];
        sc[i] = BScaleDesc{x[i], x[i], nullptr, scal_of(G, E[i]->idx) + 64, 1.0, n[i]};
    }
    gs_launch(G, gs, 1, 0.0, false, true);
    scale_launch(G, sc);
}

// ---- H_eff products ---------------------------------------------------------------------
void run_product(TtnGroup& G, int v) {
    ProductPlan& P = product_plan(G, v);
    const int sl = prod_slices(G);
    const int e0 = G.ctx->timer.mark();
    for (auto& stp : P.stages) tplan_run(G, stp, sl, T_HEFF);
    for (auto& r : P.rounds) tplan_run(G, r, sl, T_HEFF);
    G.ctx->timer.add(T_HEFF, e0, G.ctx->timer.mark());
    G.heff_flops += P.flops;
    G.matvecs += 1;
}

// ---- link tensor move v -> u (all members) -------------------------------------------------
void run_link_move(TtnGroup& G, int v, int u) {
    MovePlan& M = move_plan(G, v, u);
    const int sl = prod_slices(G);
    const int e0 = G.ctx->timer.mark();
    for (auto& stp : M.stages) tplan_run(G, stp, sl, T_ENV);
    for (auto& r : M.rounds) tplan_run(G, r, sl, T_ENV);
    tplan_run(G, M.tg, sl, T_ENV);
    comb_run(G, M.comb);
    G.ctx->timer.add(T_ENV, e0, G.ctx->timer.mark());
    const int eid = members(G)[0]->tree.edge(v, u);
    for (auto* e : members(G)) e->estore[eid].from = v;
}

// ---- excited-state projectors (LinkProjTTN) -----------------------------------------------
// Buffers: S_L the group arena (psi), S_X M's node tensors, S_A M's overlap matrices,
// S_T1 / S_T2 temporaries, S_Y the projected vector being formed.
Bases proj_bases(TtnGroup& G, tn_ttn_env* e, TtnProj& P, double* out) {
    Bases bs{};
    bs.p[S_L] = G.arena.d();
    bs.p[S_X] = P.mbuf.d();
    bs.p[S_A] = P.ebuf.d();
    bs.p[S_T1] = e->proj_t1.d();
    bs.p[S_T2] = e->proj_t2.d();
    bs.p[S_Y] = out;
    return bs;
}

struct ProjSrc {
    int buf;
    int64_t off;
};

// M[v] with the overlap matrix of every link of v but the one toward `skip` applied to its
// leg (the M side of move_linkproj_to_next! and contract, linkproj.jl:56-78 and 143-157):
// one FP64 GEMM launch per mapped leg.  The last product goes to S_Y when `out` is given.
ProjSrc proj_mapped(tn_ttn_env* e, TtnProj& P, int v, int skip, const Bases& bs, double* out) {
    const TtnTree& t = e->tree;
    cudaStream_t st = e->ctx->stream;
    std::vector<int> dims = P.mdims[v];
    const int ns = int(t.sites[v].size());
    std::vector<int> legs;
    for (size_t j = 0; j < t.nbr[v].size(); ++j)
        if (t.nbr[v][j] != skip) legs.push_back(int(j));
    ProjSrc cur{S_X, P.moff[v]};
    int tmp = 0;
    for (size_t a = 0; a < legs.size(); ++a) {
        const int j = legs[a], w = t.nbr[v][j], li = ns + j;
        const int eid = t.edge(w, v);
        TN_REQUIRE(P.efrom[eid] == w, "TTN internal: projector overlap not oriented toward the node");
        const int dout = e->dims[v][li];
        const ProjSrc dst = (a + 1 == legs.size() && out) ? ProjSrc{S_Y, 0}
                                                          : ProjSrc{tmp ? S_T2 : S_T1, 0};
        GemmPlan g;
        add_mode_tasks(g, dims, li, dout, dst.buf, dst.off,
                       {ModeIn{cur.buf, cur.off, S_A, P.eoff[eid]}}, 0);
        g.finalize(st);
        launch_gemm_f64(g, bs, st);
        dims[li] = dout;
        cur = dst;
        if (dst.buf != S_Y) tmp ^= 1;
    }
    if (out && cur.buf != S_Y) {  // no link mapped (a single-node tree): M[v] itself
        TN_CUDA(cudaMemcpyAsync(out, P.mbuf.d() + P.moff[v], size_t(vol(dims)) * 8,
                                cudaMemcpyDeviceToDevice, st));
        cur = ProjSrc{S_Y, 0};
    }
    return cur;
}

// overlap of link (v, u) on v's side: psi[v] contracted with the mapped M[v] over every leg
// but the one toward u (move_linkproj_to_next!, linkproj.jl:56-78)
void proj_move(TtnGroup& G, tn_ttn_env* e, TtnProj& P, int v, int u) {
    const TtnTree& t = e->tree;
    cudaStream_t st = e->ctx->stream;
    const Bases bs = proj_bases(G, e, P, nullptr);
    const ProjSrc y = proj_mapped(e, P, v, u, bs, nullptr);
    const auto& dp = e->dims[v];
    const int lu = t.leg_nbr(v, u);
    const int Dp = dp[lu], Dm = P.mdims[v][lu];
    const int64_t Pr = prod(dp, 0, lu), Q = prod(dp, lu + 1, int(dp.size()));
    const int eid = t.edge(v, u);
    const int64_t phi = e->node_off[v];
    GemmPlan g;
    g.add_task(S_A, P.eoff[eid], Dp, Dm, Dp, 0);
    if (Q == 1) {         // E = Phi^T Y over the rows
        g.add_seg(S_L, phi, int(Pr), 1, y.buf, y.off, int(Pr), 0, int(Pr));
    } else if (Pr == 1) { // E = Phi Y^T over the columns
        g.add_seg(S_L, phi, Dp, 0, y.buf, y.off, Dm, 1, int(Q));
    } else {              // E = sum_q Phi_q^T Y_q
        for (int64_t q = 0; q < Q; ++q)
            g.add_seg(S_L, phi + q * Pr * Dp, int(Pr), 1, y.buf, y.off + q * Pr * Dm, int(Pr), 0,
                      int(Pr));
    }
    g.finalize(st);
    launch_gemm_f64(g, bs, st);
    P.efrom[eid] = v;
}

void proj_move_all(TtnGroup& G, int v, int u) {
    const int e0 = G.ctx->timer.mark();
    bool any = false;
    for (auto* e : members(G))
        for (auto& P : e->proj) {
            proj_move(G, e, P, v, u);
            any = true;
        }
    if (any) G.ctx->timer.add(T_ENV, e0, G.ctx->timer.mark());
}

// m_k at `node` for every member with projectors (ProjTTN's contract, linkproj.jl:143-157)
void proj_vectors(TtnGroup& G, int node) {
    for (auto* e : members(G)) {
        const int64_t S = (e->S + 31) / 32 * 32;
        for (size_t k = 0; k < e->proj.size(); ++k) {
            double* out = e->proj_m.d() + int64_t(k) * S;
            proj_mapped(e, e->proj[k], node, -1, proj_bases(G, e, e->proj[k], out), out);
        }
    }
}

// y += w sum_k m_k (m_k . x) on the matvec buffers (EnvCouplingModelProjTTN's product,
// src/ttn/environment.jl:104-110)
void proj_apply(TtnGroup& G, int node) {
    for (auto* e : members(G)) {
        const int K = int(e->proj.size());
        if (K == 0) continue;
        const int64_t n = vol(e->dims[node]), S = (e->S + 31) / 32 * 32;
        std::vector<const double*> m(K);
        for (int k = 0; k < K; ++k) m[k] = e->proj_m.d() + int64_t(k) * S;
        launch_multi_dot(m.data(), K, wptr(G, e, e->w_x), n, e->proj_part.d(), e->proj_c.d(),
                         G.ctx->stream);
        launch_multi_axpy(wptr(G, e, e->w_y), m.data(), K, e->proj_c.d(), e->proj_weight, n,
                          G.ctx->stream);
    }
}

void run_product_proj(TtnGroup& G, int v) {
    run_product(G, v);
    const int e0 = G.ctx->timer.mark();
    proj_apply(G, v);
    G.ctx->timer.add(T_HEFF, e0, G.ctx->timer.mark());
}

// ---- isometry move v -> u (QR; all members) ------------------------------------------------
std::unique_ptr<QrPlan> build_qr_plan(TtnGroup& G, int v, int u, const std::vector<char>& blocked,
                                      const std::vector<int>& kmins) {
    auto slot = std::make_unique<QrPlan>();
    QrPlan& Q = *slot;
    auto E = members(G);
    const TtnTree& t = E[0]->tree;
    const int lu = t.leg_nbr(v, u), lv = t.leg_nbr(u, v);
    int npanel = 0;
    for (size_t i = 0; i < E.size(); ++i) {
        if (!blocked[i]) continue;
        const int n = E[i]->dims[v][lu];
        npanel = std::max(npanel, (n + HH_B - 1) / HH_B);
    }
    Q.npanel = npanel;
    Q.w.resize(npanel);
    Q.w2.resize(npanel);
    Q.upd.resize(npanel);
    Q.wc.resize(npanel);
    for (size_t i = 0; i < E.size(); ++i) {
        tn_ttn_env* e = E[i];
        const auto& dv = e->dims[v];
        const int n = dv[lu];
        const int64_t m = vol(dv) / n;
        const int kmin = kmins[i];
        // the factored matrix: the node tensor itself when the leg is last, else the copy
        const bool inplace = lu == int(dv.size()) - 1;
        const int abuf = inplace ? S_L : S_R;
        const int64_t aoff = inplace ? e->node_off[v] : e->wbase + e->w_qa;
        if (blocked[i]) {
            for (int p = 0; p * HH_B < kmin; ++p) {
                const int p0 = p * HH_B, pb = std::min(HH_B, kmin - p0);
                const int64_t rows = m - p0;
                const int64_t voff = e->wbase + e->w_qv + hh_panel_voff(int(m), p0);
                const int64_t toff = e->wbase + e->w_tt + int64_t(p) * HH_B * HH_B;
                const int nt = n - p0 - pb;
                if (nt > 0) {
                    // Wt = A_trail^T V (split over rows; nt x pb so that the long side is M),
                    // W2 = (-T)^T Wt^T, A_trail += V W2
                    const int64_t atr = aoff + p0 + int64_t(p0 + pb) * m;
                    const int nch = int(std::min<int64_t>(e->nchunk_q, std::max<int64_t>(1, rows / 512)));
                    const int64_t per = (rows + nch - 1) / nch;
                    std::vector<int64_t> parts;
                    for (int c = 0; c < nch; ++c) {
                        const int64_t r0 = c * per, r1 = std::min(rows, r0 + per);
                        if (r0 >= r1) break;
                        const int64_t wo = nch > 1 ? e->wbase + e->w_wp + int64_t(c) * HH_B * nt
                                                   : e->wbase + e->w_w;
                        Q.w[p].g.add_task(S_R, wo, nt, pb, nt, 0);
                        Q.w[p].g.add_seg(abuf, atr + r0, int(m), 1, S_R, voff + r0, int(m), 0,
                                         int(r1 - r0));
                        if (nch > 1) parts.push_back(wo);
                    }
                    if (parts.size() > 1) {
                        CombOut o{};
                        o.doff = e->wbase + e->w_w;
                        o.dbuf = S_R;
                        o.ldd = nt;
                        o.rows = nt;
                        o.cols = pb;
                        o.t0 = int(Q.wc[p].terms.size());
                        o.nt = int(parts.size());
                        for (int64_t po : parts) Q.wc[p].terms.push_back(CombTerm{po, S_R, nt, 1.0});
                        Q.wc[p].outs.push_back(o);
                    }
                    Q.w2[p].g.add_task(S_R, e->wbase + e->w_w2, pb, nt, pb, 0);
                    Q.w2[p].g.add_seg(S_R, toff, HH_B, 1, S_R, e->wbase + e->w_w, nt, 1, pb);
                    Q.upd[p].g.add_task(abuf, atr, int(rows), nt, int(m), 1);
                    Q.upd[p].g.add_seg(S_R, voff, int(m), 0, S_R, e->wbase + e->w_w2, pb, 0, pb);
                }
            }
            // Q formation: G = V^T V over row chunks (partials combined), W = (-T) V_top^T,
            // Q (= [I; 0] beforehand) += V W
            const int64_t vo = e->wbase + e->w_qv;
            const int64_t cap = std::max<int64_t>(1, int64_t(e->nchunk_q) * HH_B * e->dmax /
                                                         (int64_t(kmin) * kmin));
            const int nch = int(std::min<int64_t>(cap, std::max<int64_t>(1, m / 512)));
            const int64_t per = (m + nch - 1) / nch;
            std::vector<int64_t> parts;
            for (int c = 0; c < nch; ++c) {
                const int64_t r0 = c * per, r1 = std::min<int64_t>(m, r0 + per);
                if (r0 >= r1) break;
                const int64_t wo = nch > 1 ? e->wbase + e->w_wp + int64_t(c) * kmin * kmin
                                           : e->wbase + e->w_g;
                Q.gram.g.add_task(S_R, wo, kmin, kmin, kmin, 0);
                Q.gram.g.add_seg(S_R, vo + r0, int(m), 1, S_R, vo + r0, int(m), 0, int(r1 - r0));
                if (nch > 1) parts.push_back(wo);
            }
            if (parts.size() > 1) {
                CombOut o{};
                o.doff = e->wbase + e->w_g;
                o.dbuf = S_R;
                o.ldd = kmin;
                o.rows = kmin;
                o.cols = kmin;
                o.t0 = int(Q.gramc.terms.size());
                o.nt = int(parts.size());
                for (int64_t po : parts) Q.gramc.terms.push_back(CombTerm{po, S_R, kmin, 1.0});
                Q.gramc.outs.push_back(o);
            }
            Q.qw.g.add_task(S_R, e->wbase + e->w_wq, kmin, kmin, kmin, 0);
            Q.qw.g.add_seg(S_R, e->wbase + e->w_tall, kmin, 0, S_R, vo, int(m), 1, kmin);
            Q.qfin.g.add_task(abuf, aoff, int(m), kmin, int(m), 1);
            Q.qfin.g.add_seg(S_R, vo, int(m), 0, S_R, e->wbase + e->w_wq, kmin, 0, kmin);
        }
        // psi_u <- R x_lv psi_u (into the rt temporary, copied back afterwards)
        add_mode_tasks(Q.rmode.g, e->dims[u], lv, kmin, S_R, e->wbase + e->w_rt,
                       {ModeIn{S_L, e->node_off[u], S_R, e->wbase + e->w_r}}, 0);
    }
    return slot;
}

QrPlan& qr_plan(TtnGroup& G, int v, int u, const std::vector<char>& blocked,
                const std::vector<int>& kmins) {
    check_cache(G);
    auto& slot = G.qcache[{v, u}];
    if (!slot) slot = build_qr_plan(G, v, u, blocked, kmins);
    return *slot;
}

void run_qr_move(TtnGroup& G, int v, int u, int maxdim, int mindim = 1, double cutoff = -1.0) {
    auto E = members(G);
    const TtnTree& t = E[0]->tree;
    const int lu = t.leg_nbr(v, u), lv = t.leg_nbr(u, v);
    cudaStream_t st = G.ctx->stream;
    ensure_scal(G);
    const int e0 = G.ctx->timer.mark();
    std::vector<char> blocked(E.size(), 0);
    std::vector<PermDesc> to, back;
    std::vector<QrDesc> small;
    std::vector<HhDesc> hh;
    std::vector<int> kmins(E.size());
    int64_t nmax = 1, mmax = 1, mnmax = 1;
    int kmax = 0;
    std::vector<char> truncate(E.size(), 0);
    for (size_t i = 0; i < E.size(); ++i) {
        tn_ttn_env* e = E[i];
        const auto& dv = e->dims[v];
        const int n = dv[lu];
        const int64_t m = vol(dv) / n;
        const int kmin = int(std::min<int64_t>(m, n));
        kmins[i] = kmin;
        const bool inplace = lu == int(dv.size()) - 1;
        double* A = inplace ? aptr(G, e->node_off[v]) : wptr(G, e, e->w_qa);
        if (!inplace) {
            const int64_t P = prod(dv, 0, lu), Qd = prod(dv, lu + 1, int(dv.size()));
            to.push_back(PermDesc{aptr(G, e->node_off[v]), A, P, n, Qd, 1, 0});
        }
        nmax = std::max(nmax, vol(dv));
        // cutoff > 0 or a link larger than maxdim: truncating SVD move (moveisometry_to_next!,
        // ttn.jl:292-300)
        truncate[i] = n > maxdim || cutoff > 0.0;
        if (truncate[i]) continue;
        const bool blk = m * n > SMALL_QR && m >= n;
        blocked[i] = blk;
        if (!blk) {
            small.push_back(QrDesc{A, wptr(G, e, e->w_r), wptr(G, e, e->w_tau), int(m), n});
        } else {
            HhDesc h{};
            h.A = A;
            h.Q = A;
            h.R = wptr(G, e, e->w_r);
            h.V = wptr(G, e, e->w_qv);
            h.T = wptr(G, e, e->w_tt);
            h.tau = wptr(G, e, e->w_tau);
            h.scal = wptr(G, e, e->w_small);
            h.wv = wptr(G, e, e->w_small) + 16;
            h.part = wptr(G, e, e->w_hpart);
            h.G = wptr(G, e, e->w_g);
            h.Tall = wptr(G, e, e->w_tall);
            h.Yscr = wptr(G, e, e->w_wq);
            h.ticket = hh_ticket(G, e->idx);
            h.m = int(m);
            h.n = n;
            h.kmin = kmin;
            hh.push_back(h);
            mmax = std::max(mmax, m);
            mnmax = std::max(mnmax, m * n);
            kmax = std::max(kmax, kmin);
        }
    }
    if (!to.empty()) {
        upload_descs(G, G.d_perm, to);
        launch_permute(G.d_perm.as<PermDesc>(), int(to.size()), nmax, st);
    }
    for (size_t i = 0; i < E.size(); ++i) {
        if (!truncate[i]) continue;
        tn_ttn_env* e = E[i];
        const auto& dv = e->dims[v];
        const int n = dv[lu];
        const int64_t m = vol(dv) / n;
        const bool inplace = lu == int(dv.size()) - 1;
        const double* A = inplace ? aptr(G, e->node_off[v]) : wptr(G, e, e->w_qa);
        // U into the QR work (then like Q), S V^T into the R slot
        kmins[i] = svd_truncate_dense(G.ctx, A, int(m), n, maxdim, mindim, cutoff,
                                      wptr(G, e, e->w_qv), wptr(G, e, e->w_r), nullptr);
        double* dst = inplace ? aptr(G, e->node_off[v]) : wptr(G, e, e->w_qa);
        TN_CUDA(cudaMemcpyAsync(dst, wptr(G, e, e->w_qv), size_t(m) * kmins[i] * 8,
                                cudaMemcpyDeviceToDevice, st));
    }
    if (!small.empty()) {
        upload_descs(G, G.d_qr, small);
        const int q0 = G.ctx->timer.mark();
        launch_qr_small(G.d_qr.as<QrDesc>(), int(small.size()), st);
        G.ctx->timer.add(T_QRPANEL, q0, G.ctx->timer.mark());
    }
    // a truncating move changes the dimensions: its plan is built for this move only
    std::unique_ptr<QrPlan> once;
    const bool any_trunc = std::find(truncate.begin(), truncate.end(), 1) != truncate.end();
    if (any_trunc) once = build_qr_plan(G, v, u, blocked, kmins);
    QrPlan& QP = any_trunc ? *once : qr_plan(G, v, u, blocked, kmins);
    if (!hh.empty()) {
        // CTAs of the cooperative panel kernel, in proportion to the rows of each matrix
        const int cap = hh_coop_capacity();
        const int nh0 = int(hh.size());
        bool coop = nh0 <= cap;
        if (coop) {
            double tot = 0;
            for (auto& h : hh) tot += double(h.m);
            int used = 0;
            for (auto& h : hh) {
                h.ncta = std::max(1, int(double(cap - nh0) * double(h.m) / tot));
                h.ncta = int(std::min<int64_t>(h.ncta, std::max<int64_t>(1, (h.m + 255) / 256)));
                h.cta0 = used;
                used += h.ncta;
            }
            coop = used <= cap;
        }
        if (G.bars.bytes < hh.size() * sizeof(unsigned))
            G.bars.alloc(std::max<size_t>(hh.size() * sizeof(unsigned), 64), st);
        int nctas = 0;
        for (size_t i = 0; i < hh.size(); ++i) {
            hh[i].bar = G.bars.as<unsigned>() + i;
            nctas = std::max(nctas, hh[i].cta0 + hh[i].ncta);
        }
        upload_descs(G, G.d_hh, hh);
        const HhDesc* dh = G.d_hh.as<HhDesc>();
        const int nh = int(hh.size());
        const int sl = qr_slices(G);
        tn_ctx* ctx = G.ctx;
        for (int p = 0; p * HH_B < kmax; ++p) {
            const int p0 = p * HH_B, pend = p0 + HH_B;
            const int q0 = ctx->timer.mark();
            if (coop) {
                TN_CUDA(cudaMemsetAsync(G.bars.p, 0, size_t(nh) * sizeof(unsigned), st));
                launch_hh_panel_coop(dh, nh, nctas, p0, ctx->err.as<int>(), st);
            } else {
                for (int j = p0; j < std::min(pend, kmax); ++j)
                    launch_hh_column(dh, nh, mmax, j, p0, pend, st);
            }
            launch_hh_panel_end(dh, nh, mmax, p0, HH_B, st);
            const int q1 = ctx->timer.mark();
            tplan_run(G, QP.w[p], sl, T_SVD);
            comb_run(G, QP.wc[p]);
            tplan_run(G, QP.w2[p], sl, T_SVD);
            tplan_run(G, QP.upd[p], sl, T_SVD);
            ctx->timer.add(T_QRPANEL, q0, q1);
            ctx->timer.add(T_QRGEMM, q1, ctx->timer.mark());
        }
        launch_hh_finish(dh, nh, mnmax, st);
        const int q2 = ctx->timer.mark();
        tplan_run(G, QP.gram, sl, T_SVD);
        comb_run(G, QP.gramc);
        launch_hh_tall(dh, nh, st);
        tplan_run(G, QP.qw, sl, T_SVD);
        tplan_run(G, QP.qfin, sl, T_SVD);
        ctx->timer.add(T_QRGEMM, q2, ctx->timer.mark());
    }
    // Q back into the node tensor (leg lu now of size kmin)
    for (size_t i = 0; i < E.size(); ++i) {
        tn_ttn_env* e = E[i];
        auto& dv = e->dims[v];
        const bool inplace = lu == int(dv.size()) - 1;
        if (!inplace) {
            const int64_t P = prod(dv, 0, lu), Qd = prod(dv, lu + 1, int(dv.size()));
            back.push_back(PermDesc{wptr(G, e, e->w_qa), aptr(G, e->node_off[v]), P, kmins[i], Qd, 0, 0});
        }
    }
    if (!back.empty()) {
        upload_descs(G, G.d_perm, back);
        launch_permute(G.d_perm.as<PermDesc>(), int(back.size()), nmax, st);
    }
    // psi_u <- R x_lv psi_u
    tplan_run(G, QP.rmode, qr_slices(G), T_SVD);
    bool changed = false;
    for (size_t i = 0; i < E.size(); ++i) {
        tn_ttn_env* e = E[i];
        auto& du = e->dims[u];
        auto nd = du;
        nd[lv] = kmins[i];
        TN_CUDA(cudaMemcpyAsync(aptr(G, e->node_off[u]), wptr(G, e, e->w_rt), size_t(vol(nd)) * 8,
                                cudaMemcpyDeviceToDevice, st));
        if (kmins[i] != e->dims[v][lu]) changed = true;
        e->dims[v][lu] = kmins[i];
        du[lv] = kmins[i];
        e->center = u;
    }
    if (changed) G.dims_version++;
    G.ctx->timer.add(T_SVD, e0, G.ctx->timer.mark());
}

// ---- position!, update_position!, fullsweep! ---------------------------------------------
// position! (state_envs_ttn.jl:120-141): isometry moves from the centre to node (QR, or the
// truncating SVD when cutoff > 0 or a link exceeds maxdim), then the link tensors moved along
// the same path but out of `skip` (move_linktensors!'s node_to_skip, linktensors.jl:130-154)
void position_group(TtnGroup& G, int node, bool normalize, int maxdim, int mindim = 1,
                    double cutoff = -1.0, int skip = -1) {
    auto E = members(G);
    const int oc = E[0]->center;
    for (auto* e : E) TN_REQUIRE(e->center == oc, "TTN: environments of a group have different centres");
    TN_REQUIRE(oc >= 0, "TTN: the state has no orthogonality centre");
    const auto path = E[0]->tree.path(oc, node);
    for (size_t k = 0; k + 1 < path.size(); ++k)
        run_qr_move(G, path[k], path[k + 1], maxdim, mindim, cutoff);
    if (normalize) {
        std::vector<double*> x;
        std::vector<int64_t> n;
        for (auto* e : E) {
            x.push_back(aptr(G, e->node_off[node]));
            n.push_back(vol(e->dims[node]));
        }
        normalize_batch(G, E, x, n);
    }
    for (size_t k = 0; k + 1 < path.size(); ++k) {
        if (path[k] == skip) continue;
        run_link_move(G, path[k], path[k + 1]);
        proj_move_all(G, path[k], path[k + 1]);
    }
}

// Lowest eigenpair of H_eff at `node` for every member, thick-restart Lanczos in lockstep
// (KrylovKit eigsolve semantics as in the MPS engine); results replace the node tensors.
void lanczos_group(TtnGroup& G, int node, const tn_update_params* prm) {
    auto E = members(G);
    const int kd = prm->krylovdim;
    TN_REQUIRE(kd >= 1 && kd <= 16, "TTN: krylovdim must be in 1..16");
    ensure_work(G, kd);
    ensure_scal(G);
    tn_ctx* ctx = G.ctx;
    cudaStream_t st = ctx->stream;
    const size_t ni = E.size();
    struct St {
        int64_t n;
        std::vector<double*> V, pool;
        std::vector<double> Hm, D, U;
        double beta = 0;
        int numiter = 1, converged = 0, matvecs = 0;
        bool done = false;
        double& H(int i, int j, int kd) { return Hm[size_t(i) * (kd + 1) + j]; }
    };
    std::vector<St> S(ni);
    for (size_t i = 0; i < ni; ++i) {
        tn_ttn_env* e = E[i];
        S[i].n = vol(e->dims[node]);
        for (int k = 0; k < e->kry_vecs; ++k) S[i].pool.push_back(wptr(G, e, e->w_kry) + int64_t(k) * ((e->S + 31) / 32 * 32));
        S[i].Hm.assign(size_t(kd + 1) * (kd + 1), 0.0);
    }
    auto take = [&](St& s) {
        TN_REQUIRE(!s.pool.empty(), "TTN internal: Krylov pool exhausted");
        double* q = s.pool.back();
        s.pool.pop_back();
        return q;
    };
    std::vector<double> hostscal(ni * SCAL_PER);
    auto read_scal = [&]() {
        TN_CUDA(cudaMemcpyAsync(hostscal.data(), G.scal.p, ni * SCAL_PER * 8, cudaMemcpyDeviceToHost, st));
        TN_CUDA(cudaStreamSynchronize(st));
    };
    auto sc = [&](size_t i) { return scal_of(G, E[i]->idx); };
    // gs2 on the listed instances: h = V^T w twice, w -= V h, beta = |w|
    auto gs2 = [&](const std::vector<size_t>& act) {
        const int e0 = ctx->timer.mark();
        int kmax = 1;
        std::vector<BGsDesc> d(act.size());
        for (size_t a = 0; a < act.size(); ++a) {
            const size_t i = act[a];
            d[a] = BGsDesc{};
            for (size_t k = 0; k < S[i].V.size(); ++k) d[a].V[k] = S[i].V[k];
            d[a].kk = int(S[i].V.size());
            d[a].w = wptr(G, E[i], E[i]->w_y);
            d[a].n = S[i].n;
            d[a].out = sc(i);
            kmax = std::max(kmax, d[a].kk);
        }
        gs_launch(G, d, kmax, 0.0, true, false);
        for (size_t a = 0; a < act.size(); ++a) {
            d[a].hin = sc(act[a]);
            d[a].out = sc(act[a]) + 32;
        }
        gs_launch(G, d, kmax, -1.0, true, false);
        for (size_t a = 0; a < act.size(); ++a) {
            d[a].hin = sc(act[a]) + 32;
            d[a].out = sc(act[a]) + 64;
        }
        gs_launch(G, d, kmax, -1.0, false, true);
        ctx->timer.add(T_LANCZOS, e0, ctx->timer.mark());
        read_scal();
    };
    auto hvec = [&](size_t i, int K) {
        std::vector<double> h(K);
        for (int k = 0; k < K; ++k) h[k] = hostscal[i * SCAL_PER + k] + hostscal[i * SCAL_PER + 32 + k];
        S[i].beta = std::sqrt(std::max(hostscal[i * SCAL_PER + 64], 0.0));
        return h;
    };
    // V0 = x0 / |x0| (also into the matvec input)
    {
        std::vector<BGsDesc> d(ni);
        std::vector<BScaleDesc> s(ni);
        for (size_t i = 0; i < ni; ++i) {
            double* x0 = aptr(G, E[i]->node_off[node]);
            d[i] = BGsDesc{};
            d[i].w = x0;
            d[i].n = S[i].n;
            d[i].out = sc(i) + 64;
            double* v0 = take(S[i]);
            S[i].V.push_back(v0);
            s[i] = BScaleDesc{x0, v0, wptr(G, E[i], E[i]->w_x), sc(i) + 64, 1.0, S[i].n};
        }
        gs_launch(G, d, 1, 0.0, false, true);
        scale_launch(G, s);
    }
    proj_vectors(G, node);
    run_product_proj(G, node);
    for (auto& s : S) s.matvecs++;
    {
        std::vector<size_t> all(ni);
        std::iota(all.begin(), all.end(), 0);
        gs2(all);
        for (size_t i = 0; i < ni; ++i) {
            auto h = hvec(i, 1);
            S[i].H(0, 0, kd) = h[0];
        }
    }
    while (true) {
        std::vector<size_t> act, restart;
        for (size_t i = 0; i < ni; ++i) {
            St& s = S[i];
            if (s.done) continue;
            const int K = int(s.V.size());
            const bool exhausted = int64_t(K) >= s.n;
            if (K == kd || s.beta <= prm->tol || (prm->eager && K >= 1) || exhausted) {
                std::vector<double> A(size_t(K) * K);
                for (int a = 0; a < K; ++a)
                    for (int b = 0; b < K; ++b)
                        A[size_t(a) * K + b] = 0.5 * (s.H(a, b, kd) + s.H(b, a, kd));
                sym_eig_host(K, A, s.D, s.U);
                s.converged = 0;
                while (s.converged < K &&
                       std::fabs(s.beta * s.U[size_t(K - 1) * K + s.converged]) <= prm->tol)
                    s.converged++;
                if (s.converged >= 1 || exhausted) {
                    s.done = true;
                    continue;
                }
            }
            if (K < kd) {
                act.push_back(i);
            } else {
                if (s.numiter == prm->maxiter) {
                    s.done = true;
                    continue;
                }
                restart.push_back(i);
                act.push_back(i);
            }
        }
        if (act.empty()) break;
        // thick restart: keep (3 kd + 2 converged) / 5 Ritz vectors
        if (!restart.empty()) {
            std::vector<BLinDesc> d;
            std::vector<double> coefs;
            std::vector<std::pair<size_t, std::vector<double*>>> newv;
            for (size_t i : restart) {
                St& s = S[i];
                const int K = int(s.V.size());
                const int keep = (3 * kd + 2 * s.converged) / 5;
                std::vector<double> c(size_t(BK_MAX) * BK_MAX, 0.0);
                std::vector<double*> NV;
                for (int j = 0; j < keep; ++j) {
                    for (int a = 0; a < K; ++a) c[size_t(j) * BK_MAX + a] = s.U[size_t(a) * K + j];
                    double* q = take(s);
                    NV.push_back(q);
                    BLinDesc l{};
                    for (int a = 0; a < K; ++a) l.V[a] = s.V[a];
                    l.kk = K;
                    l.coef = wptr(G, E[i], E[i]->w_coef) + int64_t(j) * BK_MAX;
                    l.dst = q;
                    l.n = s.n;
                    d.push_back(l);
                }
                TN_CUDA(cudaMemcpyAsync(wptr(G, E[i], E[i]->w_coef), c.data(), c.size() * 8,
                                        cudaMemcpyHostToDevice, st));
                newv.push_back({i, NV});
            }
            const int e0 = ctx->timer.mark();
            lin_launch(G, d);
            ctx->timer.add(T_LANCZOS, e0, ctx->timer.mark());
            TN_CUDA(cudaStreamSynchronize(st));  // host coefficient arrays go out of scope
            for (auto& nv : newv) {
                St& s = S[nv.first];
                const int keep = int(nv.second.size());
                for (double* q : s.V) s.pool.push_back(q);
                s.V = nv.second;
                std::fill(s.Hm.begin(), s.Hm.end(), 0.0);
                for (int j = 0; j < keep; ++j) s.H(j, j, kd) = s.D[j];
                s.numiter++;
            }
        }
        // expansion: v = w / beta into the basis and the matvec input
        {
            std::vector<BScaleDesc> d;
            for (size_t i : act) {
                St& s = S[i];
                double* v = take(s);
                s.V.push_back(v);
                d.push_back(BScaleDesc{wptr(G, E[i], E[i]->w_y), v, wptr(G, E[i], E[i]->w_x), nullptr,
                                       1.0 / s.beta, s.n});
            }
            const int e0 = ctx->timer.mark();
            scale_launch(G, d);
            ctx->timer.add(T_LANCZOS, e0, ctx->timer.mark());
        }
        run_product_proj(G, node);
        for (size_t i : act) S[i].matvecs++;
        gs2(act);
        for (size_t i : act) {
            St& s = S[i];
            const int K = int(s.V.size());
            auto h = hvec(i, K);
            for (int a = 0; a < K; ++a) {
                s.H(a, K - 1, kd) = h[a];
                s.H(K - 1, a, kd) = h[a];
            }
        }
    }
    // Ritz vector of the lowest value, normalised, into the node tensors
    {
        std::vector<BLinDesc> d(ni);
        std::vector<double*> x(ni);
        std::vector<int64_t> n(ni);
        for (size_t i = 0; i < ni; ++i) {
            St& s = S[i];
            const int K = int(s.V.size());
            std::vector<double> c(K);
            for (int a = 0; a < K; ++a) c[a] = s.U[size_t(a) * K + 0];
            TN_CUDA(cudaMemcpyAsync(wptr(G, E[i], E[i]->w_coef), c.data(), K * 8, cudaMemcpyHostToDevice, st));
            d[i] = BLinDesc{};
            for (int a = 0; a < K; ++a) d[i].V[a] = s.V[a];
            d[i].kk = K;
            d[i].coef = wptr(G, E[i], E[i]->w_coef);
            d[i].dst = aptr(G, E[i]->node_off[node]);
            d[i].n = s.n;
            x[i] = d[i].dst;
            n[i] = s.n;
        }
        lin_launch(G, d);
        normalize_batch(G, E, x, n);
        TN_CUDA(cudaStreamSynchronize(st));
    }
    for (size_t i = 0; i < ni; ++i) {
        E[i]->energy = S[i].D[0];
        E[i]->matvecs = S[i].matvecs;
        E[i]->converged = S[i].converged;
    }
}

void check_ttn_params(const tn_update_params* p, bool allow_noise = false) {
    TN_REQUIRE(p != nullptr, "null parameters");
    TN_REQUIRE(allow_noise || p->noise == 0.0,
               "TTN: noise > 0 takes the subspace-expansion sweep (tn_ttn_envs_fullsweep_expand)");
    TN_REQUIRE(p->maxiter >= 1 && p->krylovdim >= 1, "bad solver parameters");
}

void update_group(TtnGroup& G, int node, const tn_update_params* p, double cutoff = -1.0) {
    check_ttn_params(p, true);
    ensure_work(G, p->krylovdim);
    position_group(G, node, p->normalize != 0, p->maxdim, std::max(1, p->mindim), cutoff);
    lanczos_group(G, node, p);
    if (p->check_convergence)
        for (auto* e : members(G))
            if (e->converged < 1) throw Error(TN_E_NOTCONV, "eigsolve did not converge");
}

int maxlinkdim_of(const TtnTree& t, const std::vector<std::vector<int>>& dims) {
    int md = 1;
    for (int v = 0; v < t.nn; ++v)
        for (size_t j = 0; j < t.nbr[v].size(); ++j) md = std::max(md, dims[v][t.sites[v].size() + j]);
    return md;
}

void collect_stats(TtnGroup& G) {
    TN_CUDA(cudaStreamSynchronize(G.ctx->stream));
    G.ctx->timer.collect(G.acc_ms);
}

void reset_stats(TtnGroup& G) {
    collect_stats(G);
    std::fill(G.acc_ms, G.acc_ms + T_NCAT, 0.0);
    G.heff_flops = G.gemm_flops = G.krylov_bytes = 0;
    G.gemm_launches = G.matvecs = 0;
}

// LinkTensorsTTN(psi, M): link tensors from the leaves toward the centre
void build_links(TtnGroup& G) {
    auto E = members(G);
    const int oc = E[0]->center;
    const auto order = bfs_reverse(E[0]->tree, oc);
    for (int v : order) {
        if (v == oc) continue;
        const auto path = E[0]->tree.path(v, oc);
        run_link_move(G, v, path[1]);
    }
}

std::unique_ptr<tn_ttn> copy_out(TtnGroup& G, tn_ttn_env* e) {
    auto p = std::make_unique<tn_ttn>();
    p->ctx = e->ctx;
    p->tree = e->tree;
    p->dims = e->dims;
    p->center = e->center;
    p->node.resize(e->tree.nn);
    for (int v = 0; v < e->tree.nn; ++v) {
        const int64_t n = vol(e->dims[v]);
        p->node[v].alloc(size_t(n) * 8, e->ctx->stream);
        TN_CUDA(cudaMemcpyAsync(p->node[v].p, aptr(G, e->node_off[v]), size_t(n) * 8,
                                cudaMemcpyDeviceToDevice, e->ctx->stream));
    }
    TN_CUDA(cudaStreamSynchronize(e->ctx->stream));
    return p;
}

}  // namespace

// -------------------------------------------------------------------------------------
// C ABI
// -------------------------------------------------------------------------------------
namespace {

void upload_site_ops(TtnGroup& G, tn_ttn_env* e);

std::shared_ptr<TtnGroup> make_group(tn_ctx* ctx, const std::vector<const tn_ttn*>& psis,
                                     const std::vector<const tn_ttn_model*>& models,
                                     std::vector<tn_ttn_env*>& out) {
    TN_REQUIRE(!psis.empty(), "TTN: no states");
    auto G = std::make_shared<TtnGroup>();
    G->ctx = ctx;
    const tn_ttn* p0 = psis[0];
    int64_t cursor = 0;
    std::vector<std::unique_ptr<tn_ttn_env>> envs;
    for (size_t i = 0; i < psis.size(); ++i) {
        const tn_ttn* p = psis[i];
        TN_REQUIRE(p && p->ctx == ctx, "TTN: states of one group need one context");
        TN_REQUIRE(p->tree.N == p0->tree.N && p->tree.nn == p0->tree.nn && p->tree.d == p0->tree.d &&
                       p->tree.edges == p0->tree.edges && p->tree.site_node == p0->tree.site_node,
                   "TTN: states of one group need one tree");
        TN_REQUIRE(p->center >= 0 && p->center == p0->center,
                   "TTN: states of one group need one orthogonality centre");
        const tn_ttn_model* m = models[i];
        TN_REQUIRE(m && m->N == p->tree.N && m->d == p->tree.d, "TTN: model does not match the sites");
        auto e = std::make_unique<tn_ttn_env>();
        e->grp = G;
        e->idx = int(i);
        e->ctx = ctx;
        e->tree = p->tree;
        e->model = *m;
        e->dims = p->dims;
        e->center = p->center;
        build_arena_layout(e.get(), cursor);
        envs.push_back(std::move(e));
    }
    cudaStream_t st = ctx->stream;
    G->arena.alloc(size_t(std::max<int64_t>(cursor, 32)) * 8, st);
    TN_CUDA(cudaMemsetAsync(G->arena.p, 0, G->arena.bytes, st));
    for (size_t i = 0; i < envs.size(); ++i) {
        tn_ttn_env* e = envs[i].get();
        G->envs.push_back(e);
        const tn_ttn* p = psis[i];
        for (int v = 0; v < e->tree.nn; ++v)
            TN_CUDA(cudaMemcpyAsync(aptr(*G, e->node_off[v]), p->node[v].p,
                                    size_t(vol(e->dims[v])) * 8, cudaMemcpyDeviceToDevice, st));
        upload_site_ops(*G, e);  // local sums and per-term operators
    }
    G->alive = int(envs.size());
    ensure_work(*G, 5);
    ensure_scal(*G);
    build_links(*G);
    reset_stats(*G);
    for (auto& e : envs) out.push_back(e.release());
    return G;
}

TtnGroup& solo(tn_ttn_env* env) {
    TN_REQUIRE(env && env->grp, "null TTN environment");
    TN_REQUIRE(env->grp->alive == 1,
               "TTN: this environment belongs to a group of several; sweep the group with "
               "tn_ttn_envs_fullsweep");
    return *env->grp;
}

void fill_sweep_result(TtnGroup& G, tn_ttn_env* e, tn_sweep_result* r, int64_t launches) {
    std::memset(r, 0, sizeof(*r));
    r->energy = e->energy;
    r->maxtruncerr = 0.0;
    r->maxlinkdim = maxlinkdim_of(e->tree, e->dims);
    r->matvecs = int32_t(G.matvecs);
    r->heff_flops = G.heff_flops;
    r->heff_ms = G.acc_ms[T_HEFF];
    r->env_ms = G.acc_ms[T_ENV];
    r->svd_ms = G.acc_ms[T_SVD];
    r->lanczos_ms = G.acc_ms[T_LANCZOS];
    r->sweep_ms = G.acc_ms[T_SWEEP];
    r->gemm_ms = G.acc_ms[T_GEMM];
    r->gemm_flops = G.gemm_flops;
    r->pack_ms = G.acc_ms[T_PACK];
    r->gemm_launches = G.gemm_launches;
    r->kernel_launches = launches;
    r->qr_panel_ms = G.acc_ms[T_QRPANEL];
    r->qr_gemm_ms = G.acc_ms[T_QRGEMM];
    r->krylov_bytes = G.krylov_bytes;
}

// Overlap slots, temporaries and projected-vector buffers of every projector of e, sized
// by the slot capacities of psi (link dimensions only grow through grow_group, which calls
// this again), and the overlaps rebuilt from the leaves toward the centre (LinkProjTTN,
// linkproj.jl:188-224).
void proj_layout_and_build(TtnGroup& G, tn_ttn_env* e) {
    if (e->proj.empty()) return;
    cudaStream_t st = e->ctx->stream;
    const TtnTree& t = e->tree;
    auto r32 = [](int64_t n) { return (n + 31) / 32 * 32; };
    auto cap_of_leg = [&](int v, int l) {
        const int ns = int(t.sites[v].size());
        if (l < ns) return e->dims[v][size_t(l)];
        return std::max(e->dims[v][size_t(l)], e->estore[t.edge(v, t.nbr[v][l - ns])].cap_dim);
    };
    int64_t tn = 32;
    for (auto& P : e->proj) {
        for (int v = 0; v < t.nn; ++v) {
            // a temporary holds M[v] with any subset of its links mapped to psi's dimensions
            int64_t big = 1;
            for (size_t l = 0; l < P.mdims[v].size(); ++l)
                big *= std::max(P.mdims[v][l], cap_of_leg(v, int(l)));
            tn = std::max(tn, big);
        }
        int64_t c = 0;
        P.eoff.assign(t.edges.size(), 0);
        for (size_t ei = 0; ei < t.edges.size(); ++ei) {
            const int a = t.edges[ei].first, b = t.edges[ei].second;
            const int la = t.leg_nbr(a, b);
            P.eoff[ei] = c;
            c += r32(int64_t(cap_of_leg(a, la)) * P.mdims[a][la]);
        }
        P.ebuf.alloc(size_t(std::max<int64_t>(c, 32)) * 8, st);
        TN_CUDA(cudaMemsetAsync(P.ebuf.p, 0, P.ebuf.bytes, st));
        P.efrom.assign(t.edges.size(), -1);
    }
    const int count = int(e->proj.size());
    e->proj_tn = tn;
    e->proj_t1.alloc(size_t(tn) * 8, st);
    e->proj_t2.alloc(size_t(tn) * 8, st);
    e->proj_m.alloc(size_t(count) * r32(e->S) * 8, st);
    e->proj_c.alloc(64 * 8, st);
    e->proj_part.alloc(size_t(count) * blas_nparts() * 8, st);
    const int oc = e->center;
    for (int v : bfs_reverse(t, oc)) {
        if (v == oc) continue;
        const int next = t.path(v, oc)[1];
        for (auto& P : e->proj) proj_move(G, e, P, v, next);
    }
    TN_CUDA(cudaStreamSynchronize(st));
}

// StateEnvsTTN(psi, H, Ms; weight) (src/ttn/state_envs_ttn.jl:36-52): copies of the Ms and
// their overlaps built from the leaves toward the centre (LinkProjTTN, linkproj.jl:188-224)
void proj_setup(TtnGroup& G, tn_ttn_env* e, const tn_ttn* const* Ms, int count, double weight) {
    cudaStream_t st = e->ctx->stream;
    const TtnTree& t = e->tree;
    TN_CUDA(cudaStreamSynchronize(st));
    e->proj.clear();
    e->proj_weight = count > 0 ? weight : 0.0;
    if (count == 0) return;
    auto r32 = [](int64_t n) { return (n + 31) / 32 * 32; };
    for (int k = 0; k < count; ++k) {
        const tn_ttn* M = Ms[k];
        TtnProj P;
        P.mdims = M->dims;
        P.moff.assign(t.nn, 0);
        int64_t c = 0;
        for (int v = 0; v < t.nn; ++v) {
            P.moff[v] = c;
            c += r32(vol(M->dims[v]));
        }
        P.mbuf.alloc(size_t(std::max<int64_t>(c, 32)) * 8, st);
        for (int v = 0; v < t.nn; ++v)
            TN_CUDA(cudaMemcpyAsync(P.mbuf.d() + P.moff[v], M->node[v].p,
                                    size_t(vol(M->dims[v])) * 8, cudaMemcpyDeviceToDevice, st));
        e->proj.push_back(std::move(P));
    }
    proj_layout_and_build(G, e);
}

// site operators of an instance into its arena slots: per site the sum of its one-site terms
// (local) and the operator of every longer term (open)
void upload_site_ops(TtnGroup& G, tn_ttn_env* e) {
    cudaStream_t st = G.ctx->stream;
    const int dd = e->tree.d * e->tree.d;
    std::vector<std::vector<double>> loc(e->tree.N);
    for (size_t ti = 0; ti < e->model.terms.size(); ++ti) {
        const auto& tm = e->model.terms[ti];
        for (size_t j = 0; j < tm.sites.size(); ++j) {
            const int s = tm.sites[j];
            if (tm.sites.size() == 1) {
                if (loc[s].empty()) loc[s].assign(dd, 0.0);
                for (int k = 0; k < dd; ++k) loc[s][k] += tm.ops[j][k];
            } else {
                TN_CUDA(cudaMemcpyAsync(aptr(G, e->sstore[s].open.at(int(ti))), tm.ops[j].data(),
                                        dd * 8, cudaMemcpyHostToDevice, st));
            }
        }
    }
    for (int s = 0; s < e->tree.N; ++s)
        if (!loc[s].empty())
            TN_CUDA(cudaMemcpyAsync(aptr(G, e->sstore[s].local), loc[s].data(), dd * 8,
                                    cudaMemcpyHostToDevice, st));
    TN_CUDA(cudaStreamSynchronize(st));  // host operator copies go out of scope
}

// ---- subspace expansion (noise > 0) -------------------------------------------------------
// The arena re-laid with room for larger tensors: node slots of node_cap[i][v] elements and
// link slots of link dimension link_cap[i][e] (at least the current sizes); node tensors are
// copied over, site operators re-uploaded, link tensors and projector overlaps rebuilt from
// the leaves toward the centre, plans and work buffers dropped.
void grow_group(TtnGroup& G, const std::vector<std::vector<int64_t>>& node_cap,
                const std::vector<std::vector<int>>& link_cap) {
    auto E = members(G);
    cudaStream_t st = G.ctx->stream;
    TN_CUDA(cudaStreamSynchronize(st));
    std::vector<std::vector<int64_t>> old_off(E.size());
    int64_t cursor = 0;
    for (size_t i = 0; i < E.size(); ++i) {
        tn_ttn_env* e = E[i];
        old_off[i] = e->node_off;
        e->node_cap = node_cap[i];
        e->link_cap = link_cap[i];
        build_arena_layout(e, cursor);  // link slots re-laid: their tensors are rebuilt below
    }
    DevBuf na;
    na.alloc(size_t(std::max<int64_t>(cursor, 32)) * 8, st);
    TN_CUDA(cudaMemsetAsync(na.p, 0, na.bytes, st));
    for (size_t i = 0; i < E.size(); ++i) {
        tn_ttn_env* e = E[i];
        for (int v = 0; v < e->tree.nn; ++v)
            TN_CUDA(cudaMemcpyAsync(na.d() + e->node_off[v], G.arena.d() + old_off[i][v],
                                    size_t(vol(e->dims[v])) * 8, cudaMemcpyDeviceToDevice, st));
    }
    TN_CUDA(cudaStreamSynchronize(st));
    G.arena = std::move(na);
    for (auto* e : E) upload_site_ops(G, e);
    G.work_kd = 0;  // work layouts depend on the slot sizes
    ensure_work(G, 5);
    ensure_scal(G);
    G.dims_version++;
    check_cache(G);
    build_links(G);
    for (auto* e : E) proj_layout_and_build(G, e);
}

// dimension of the largest meaningful state space on one side of edge ei: d^(sites), capped
int full_link_dim(const TtnTree& t, int ei) {
    const auto side = t.side(t.edges[ei].first, t.edges[ei].second);
    int na = 0;
    for (char c : side) na += c ? 1 : 0;
    const int nmin = std::min(na, t.N - na);
    int64_t f = 1;
    for (int k = 0; k < nmin && f < (int64_t(1) << 30); ++k) f *= t.d;
    return int(std::min<int64_t>(f, int64_t(1) << 30));
}

// Capacity for a noisy sweep at maxdim with expansions of up to mx: every link up to
// max(current, min(maxdim, full)) and one link of a node more by mx (after each expansion
// the truncating moves bring that link back to maxdim before the next one grows).
void ensure_expand_capacity(TtnGroup& G, int maxdim, int mx) {
    auto E = members(G);
    bool grow = false;
    std::vector<std::vector<int64_t>> ncap(E.size());
    std::vector<std::vector<int>> lcap(E.size());
    for (size_t i = 0; i < E.size(); ++i) {
        tn_ttn_env* e = E[i];
        const TtnTree& t = e->tree;
        std::vector<int> c(t.edges.size());
        lcap[i].resize(t.edges.size());
        for (size_t ei = 0; ei < t.edges.size(); ++ei) {
            const int a = t.edges[ei].first, b = t.edges[ei].second;
            const int cur = e->dims[a][t.leg_nbr(a, b)];
            c[ei] = std::max(cur, std::min(maxdim, full_link_dim(t, int(ei))));
            lcap[i][ei] = std::max(e->estore[ei].cap_dim, int(std::min<int64_t>(
                                                              int64_t(c[ei]) + mx, INT_MAX)));
            grow = grow || lcap[i][ei] > e->estore[ei].cap_dim;
        }
        ncap[i].resize(t.nn);
        for (int v = 0; v < t.nn; ++v) {
            const int ns = int(t.sites[v].size());
            std::vector<int64_t> leg(size_t(t.nlegs(v)));
            for (int l = 0; l < t.nlegs(v); ++l)
                leg[l] = l < ns ? t.d : c[t.edge(v, t.nbr[v][l - ns])];
            int64_t need = vol(e->dims[v]);
            for (int l = ns; l < t.nlegs(v); ++l) {
                double prodv = 1.0;
                for (int l2 = 0; l2 < t.nlegs(v); ++l2) prodv *= double(l2 == l ? leg[l2] + mx : leg[l2]);
                TN_REQUIRE(prodv < 4e9, "TTN: subspace expansion needs a node tensor too large "
                                        "for this engine (lower maxdim or max_expand_dim)");
                need = std::max(need, int64_t(prodv));
            }
            const int64_t have = e->node_cap[size_t(v)];
            ncap[i][v] = std::max(need, have);
            grow = grow || need > have;
        }
    }
    if (grow) grow_group(G, ncap, lcap);
}

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// subspace_expand! (src/ttn/update_site_ttn.jl:75-109) of the link (node, nxt) in every
// member: the link grows by pad = min(sum of the other leg dims of each tensor,
// max_expand_dim) (indexintersection, src/base/helper_internal_funcs.jl:182-188); each tensor
// gets a random block along it scaled to noise * its norm (direct sum, old components
// first).  The padding is the counter-based stream value j = top 53 bits of
// splitmix64(key + j) mapped to [-1, 1), key = splitmix64(seed + 2 (4096 event + instance) +
// which), drawn on the host (which: 0 for node, 1 for nxt).
void expand_group(TtnGroup& G, int node, int nxt, int mx, double noise, uint64_t seed) {
    auto E = members(G);
    const TtnTree& t = E[0]->tree;
    const int la = t.leg_nbr(node, nxt), lb = t.leg_nbr(nxt, node);
    cudaStream_t st = G.ctx->stream;
    ensure_scal(G);
    std::vector<BGsDesc> ga(E.size()), gb(E.size());
    for (size_t i = 0; i < E.size(); ++i) {
        tn_ttn_env* e = E[i];
        ga[i] = BGsDesc{};
        ga[i].w = aptr(G, e->node_off[node]);
        ga[i].out = scal_of(G, e->idx) + 66;
        ga[i].n = vol(e->dims[node]);
        gb[i] = BGsDesc{};
        gb[i].w = aptr(G, e->node_off[nxt]);
        gb[i].out = scal_of(G, e->idx) + 67;
        gb[i].n = vol(e->dims[nxt]);
    }
    gs_launch(G, ga, 1, 0.0, false, true);
    gs_launch(G, gb, 1, 0.0, false, true);
    std::vector<double> hs(G.envs.size() * SCAL_PER);
    TN_CUDA(cudaMemcpyAsync(hs.data(), G.scal.p, hs.size() * 8, cudaMemcpyDeviceToHost, st));
    TN_CUDA(cudaStreamSynchronize(st));
    std::vector<double> host;
    struct Pend {
        ConcatDesc d;
        int64_t off;
    };
    std::vector<Pend> pend;
    std::vector<std::pair<tn_ttn_env*, int>> grown;
    int64_t nmax = 1;
    for (tn_ttn_env* e : E) {
        const auto& dA = e->dims[node];
        const auto& dB = e->dims[nxt];
        int64_t sa = 0, sb = 0;
        for (size_t l = 0; l < dA.size(); ++l) sa += int(l) == la ? 0 : dA[l];
        for (size_t l = 0; l < dB.size(); ++l) sb += int(l) == lb ? 0 : dB[l];
        const int pad = int(std::min<int64_t>(std::min(sa, sb), mx));
        if (pad <= 0) continue;
        for (int which = 0; which < 2; ++which) {
            const int v = which ? nxt : node, leg = which ? lb : la;
            const auto& dv = e->dims[v];
            const int64_t P = prod(dv, 0, leg), D = dv[leg], Q = prod(dv, leg + 1, int(dv.size()));
            const int64_t np = P * pad * Q;
            TN_REQUIRE(P * (D + pad) * Q <= e->node_cap[size_t(v)],
                       "TTN internal: no room for the subspace expansion");
            const uint64_t key = splitmix64(seed + uint64_t(2) * (uint64_t(4096) * uint64_t(e->expand_events) +
                                                                 uint64_t(e->idx)) + uint64_t(which));
            const int64_t off = int64_t(host.size());
            double n2 = 0.0;
            for (int64_t j = 0; j < np; ++j) {
                const double x = double(splitmix64(key + uint64_t(j)) >> 11) * 0x1p-52 - 1.0;
                host.push_back(x);
                n2 += x * x;
            }
            const double tn2 = hs[size_t(e->idx) * SCAL_PER + 66 + which];
            const double scale = n2 > 0.0 ? noise * std::sqrt(std::max(tn2, 0.0)) / std::sqrt(n2) : 0.0;
            for (int64_t j = 0; j < np; ++j) host[size_t(off + j)] *= scale;
            // the old tensor to a work temporary, then the direct sum into the node slot
            double* tmp = wptr(G, e, which ? e->w_rt : e->w_qa);
            TN_CUDA(cudaMemcpyAsync(tmp, aptr(G, e->node_off[v]), size_t(vol(dv)) * 8,
                                    cudaMemcpyDeviceToDevice, st));
            pend.push_back(Pend{ConcatDesc{tmp, nullptr, aptr(G, e->node_off[v]), P, D, pad, Q}, off});
            nmax = std::max(nmax, P * (D + pad) * Q);
        }
        grown.push_back({e, pad});
    }
    for (tn_ttn_env* e : E) e->expand_events++;
    if (pend.empty()) return;
    G.pads.alloc(std::max<size_t>(host.size(), 1) * 8, st);
    TN_CUDA(cudaMemcpyAsync(G.pads.p, host.data(), host.size() * 8, cudaMemcpyHostToDevice, st));
    std::vector<ConcatDesc> cd;
    for (auto& pd : pend) {
        pd.d.b = G.pads.d() + pd.off;
        cd.push_back(pd.d);
    }
    upload_descs(G, G.d_cat, cd);
    launch_concat(G.d_cat.as<ConcatDesc>(), int(cd.size()), nmax, st);
    for (auto& gp : grown) {
        gp.first->dims[node][la] += gp.second;
        gp.first->dims[nxt][lb] += gp.second;
    }
    G.dims_version++;
    TN_CUDA(cudaStreamSynchronize(st));  // the host padding goes out of scope
}

// fullsweep!'s noise > 0 branch (src/ttn/sweep_ttn.jl:180-243): every node of path and of the
// reversed path but the central one is expanded toward the central node, then updated
// expand_numiter times alternately with its next node
void fullsweep_expand(TtnGroup& G, const std::vector<int>& path, const tn_update_params* p,
                      int central, int expand_dim, int mx, int numiter, uint64_t seed) {
    const TtnTree& t = members(G)[0]->tree;
    ensure_expand_capacity(G, p->maxdim, mx);
    std::vector<int> order(path);
    order.insert(order.end(), path.rbegin(), path.rend());
    for (int node : order) {
        if (node == central) {
            update_group(G, node, p);
            continue;
        }
        const int nxt = t.path(node, central)[1];
        ensure_work(G, p->krylovdim);
        position_group(G, node, p->normalize != 0, p->maxdim, std::max(1, p->mindim), -1.0, nxt);
        expand_group(G, node, nxt, mx, p->noise, seed);
        for (auto* e : members(G)) e->center = nxt;
        for (int it = 1; it <= numiter; ++it) {
            tn_update_params q = *p;
            const int64_t md = it == numiter ? p->maxdim
                               : int64_t(p->maxdim) + (it == 1 ? mx : expand_dim);
            q.maxdim = int(std::min<int64_t>(md, INT_MAX));
            update_group(G, it % 2 == 1 ? node : nxt, &q, p->cutoff);
        }
    }
}

}  // namespace

extern "C" {

int tn_ttn_create(tn_ctx* ctx, int nsites, int d, int nnodes, int nedges, const int32_t* edges,
                  const int32_t* site_node, const int32_t* link_dims, const double* data,
                  int center, tn_ttn** out) {
    return guarded([&] {
        TN_REQUIRE(ctx && out && edges && site_node && link_dims && data, "null argument");
        auto p = std::make_unique<tn_ttn>();
        p->ctx = ctx;
        p->tree = make_tree(nsites, d, nnodes, nedges, edges, site_node);
        TN_REQUIRE(center >= -1 && center < nnodes, "TTN: bad centre");
        p->center = center;
        p->dims.assign(nnodes, {});
        for (int v = 0; v < nnodes; ++v) {
            for (size_t i = 0; i < p->tree.sites[v].size(); ++i) p->dims[v].push_back(d);
            for (int u : p->tree.nbr[v]) {
                // link_dims are given in the caller's edge order
                int dim = -1;
                for (int e = 0; e < nedges; ++e)
                    if ((edges[2 * e] == v && edges[2 * e + 1] == u) ||
                        (edges[2 * e] == u && edges[2 * e + 1] == v))
                        dim = link_dims[e];
                TN_REQUIRE(dim >= 1, "TTN: link dimensions must be positive");
                p->dims[v].push_back(dim);
            }
        }
        p->node.resize(nnodes);
        int64_t off = 0;
        for (int v = 0; v < nnodes; ++v) {
            const int64_t n = vol(p->dims[v]);
            p->node[v].alloc(size_t(n) * 8, ctx->stream);
            TN_CUDA(cudaMemcpyAsync(p->node[v].p, data + off, size_t(n) * 8, cudaMemcpyHostToDevice,
                                    ctx->stream));
            off += n;
        }
        TN_CUDA(cudaStreamSynchronize(ctx->stream));
        *out = p.release();
    });
}

int tn_ttn_destroy(tn_ttn* psi) {
    return guarded([&] {
        if (!psi) return;
        cudaStreamSynchronize(psi->ctx->stream);
        delete psi;
    });
}

int tn_ttn_center(const tn_ttn* psi) { return psi ? psi->center : TN_E_INVALID; }

int tn_ttn_node_dims(const tn_ttn* psi, int node, int32_t* nlegs, int32_t* dims) {
    return guarded([&] {
        TN_REQUIRE(psi && nlegs && node >= 0 && node < psi->tree.nn, "bad node");
        *nlegs = int32_t(psi->dims[node].size());
        if (dims) {
            TN_REQUIRE(psi->dims[node].size() <= 64, "too many legs");
            for (size_t i = 0; i < psi->dims[node].size(); ++i) dims[i] = psi->dims[node][i];
        }
    });
}

int tn_ttn_node(const tn_ttn* psi, int node, double* out, int64_t cap) {
    return guarded([&] {
        TN_REQUIRE(psi && out && node >= 0 && node < psi->tree.nn, "bad node");
        const int64_t n = vol(psi->dims[node]);
        TN_REQUIRE(cap >= n, "output buffer too small");
        TN_CUDA(cudaMemcpyAsync(out, psi->node[node].p, size_t(n) * 8, cudaMemcpyDeviceToHost,
                                psi->ctx->stream));
        TN_CUDA(cudaStreamSynchronize(psi->ctx->stream));
    });
}

int tn_ttn_maxlinkdim(const tn_ttn* psi) {
    if (!psi) return TN_E_INVALID;
    return maxlinkdim_of(psi->tree, psi->dims);
}

int tn_ttn_isometrize(tn_ttn* psi, int node, int normalize) {
    return guarded([&] {
        TN_REQUIRE(psi && node >= 0 && node < psi->tree.nn, "bad node");
        // a group of one with an empty model carries the QR moves
        tn_ttn_model empty;
        empty.N = psi->tree.N;
        empty.d = psi->tree.d;
        auto G = std::make_shared<TtnGroup>();
        G->ctx = psi->ctx;
        auto e = std::make_unique<tn_ttn_env>();
        e->grp = G;
        e->ctx = psi->ctx;
        e->tree = psi->tree;
        e->model = empty;
        e->dims = psi->dims;
        e->center = psi->center;
        int64_t cursor = 0;
        build_arena_layout(e.get(), cursor);
        cudaStream_t st = psi->ctx->stream;
        G->arena.alloc(size_t(std::max<int64_t>(cursor, 32)) * 8, st);
        for (int v = 0; v < psi->tree.nn; ++v)
            TN_CUDA(cudaMemcpyAsync(aptr(*G, e->node_off[v]), psi->node[v].p,
                                    size_t(vol(e->dims[v])) * 8, cudaMemcpyDeviceToDevice, st));
        G->envs.push_back(e.get());
        G->alive = 1;
        ensure_work(*G, 1);
        ensure_scal(*G);
        const int big = INT_MAX;
        if (psi->center < 0) {
            const auto order = bfs_reverse(psi->tree, node);
            for (int v : order) {
                if (v == node) continue;
                run_qr_move(*G, v, psi->tree.path(v, node)[1], big);
            }
        } else {
            const auto path = psi->tree.path(psi->center, node);
            for (size_t k = 0; k + 1 < path.size(); ++k) run_qr_move(*G, path[k], path[k + 1], big);
        }
        e->center = node;
        if (normalize) normalize_batch(*G, {e.get()}, {aptr(*G, e->node_off[node])}, {vol(e->dims[node])});
        for (int v = 0; v < psi->tree.nn; ++v) {
            const int64_t n = vol(e->dims[v]);
            if (n != vol(psi->dims[v])) psi->node[v].alloc(size_t(n) * 8, st);
            TN_CUDA(cudaMemcpyAsync(psi->node[v].p, aptr(*G, e->node_off[v]), size_t(n) * 8,
                                    cudaMemcpyDeviceToDevice, st));
        }
        psi->dims = e->dims;
        psi->center = node;
        TN_CUDA(cudaStreamSynchronize(st));
        G->envs.clear();
        check_device_error_public(psi->ctx);
    });
}

int tn_ttn_model_create(int nsites, int d, int nterms, const int32_t* term_nops,
                        const int32_t* term_sites, const double* ops, const double* coef,
                        tn_ttn_model** out) {
    return guarded([&] {
        TN_REQUIRE(out && nsites >= 1 && d >= 1 && nterms >= 0, "bad model arguments");
        auto m = std::make_unique<tn_ttn_model>();
        m->N = nsites;
        m->d = d;
        int64_t so = 0, oo = 0;
        const int dd = d * d;
        for (int t = 0; t < nterms; ++t) {
            const int k = term_nops[t];
            TN_REQUIRE(k >= 1, "a term needs at least one operator");
            std::vector<std::pair<int, std::vector<double>>> f;
            for (int j = 0; j < k; ++j) {
                const int s = term_sites[so + j];
                TN_REQUIRE(s >= 0 && s < nsites, "term site out of range");
                f.push_back({s, std::vector<double>(ops + oo + int64_t(j) * dd, ops + oo + int64_t(j + 1) * dd)});
            }
            so += k;
            oo += int64_t(k) * dd;
            std::sort(f.begin(), f.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
            for (int j = 1; j < k; ++j)
                TN_REQUIRE(f[j].first != f[j - 1].first, "a term acts twice on one site");
            tn_ttn_model::Term tm;
            for (auto& x : f) {
                tm.sites.push_back(x.first);
                tm.ops.push_back(std::move(x.second));
            }
            for (double& x : tm.ops[0]) x *= coef[t];
            m->terms.push_back(std::move(tm));
        }
        *out = m.release();
    });
}

int tn_ttn_model_destroy(tn_ttn_model* model) {
    delete model;
    return TN_OK;
}

int tn_ttn_envs_create(int count, tn_ttn* const* psis, tn_ttn_model* const* models,
                       tn_ttn_env** out) {
    return guarded([&] {
        TN_REQUIRE(count >= 1 && psis && models && out, "bad arguments");
        std::vector<const tn_ttn*> p(psis, psis + count);
        std::vector<const tn_ttn_model*> m(models, models + count);
        TN_REQUIRE(p[0] != nullptr, "null state");
        std::vector<tn_ttn_env*> envs;
        make_group(p[0]->ctx, p, m, envs);
        for (int i = 0; i < count; ++i) out[i] = envs[i];
    });
}

int tn_ttn_env_destroy(tn_ttn_env* env) {
    return guarded([&] {
        if (!env) return;
        auto G = env->grp;
        cudaStreamSynchronize(env->ctx->stream);
        G->envs[env->idx] = nullptr;
        G->alive--;
        G->pcache.clear();
        G->mcache.clear();
        G->qcache.clear();
        delete env;
    });
}

int tn_ttn_env_getpsi(tn_ttn_env* env, tn_ttn** out) {
    return guarded([&] {
        TN_REQUIRE(env && out, "null argument");
        *out = copy_out(*env->grp, env).release();
    });
}

int tn_ttn_env_center(const tn_ttn_env* env) { return env ? env->center : TN_E_INVALID; }

int tn_ttn_env_position(tn_ttn_env* env, int node) {
    return guarded([&] {
        TtnGroup& G = solo(env);
        TN_REQUIRE(node >= 0 && node < env->tree.nn, "bad node");
        position_group(G, node, true, INT_MAX);
        collect_stats(G);
        check_device_error_public(env->ctx);
    });
}

int tn_ttn_env_product(tn_ttn_env* env, const double* v, double* out, int64_t n) {
    return guarded([&] {
        TtnGroup& G = solo(env);
        TN_REQUIRE(v && out, "null argument");
        const int c = env->center;
        TN_REQUIRE(n == vol(env->dims[c]), "vector size does not match the centre tensor");
        cudaStream_t st = env->ctx->stream;
        TN_CUDA(cudaMemcpyAsync(wptr(G, env, env->w_x), v, size_t(n) * 8, cudaMemcpyHostToDevice, st));
        proj_vectors(G, c);
        run_product_proj(G, c);
        TN_CUDA(cudaMemcpyAsync(out, wptr(G, env, env->w_y), size_t(n) * 8, cudaMemcpyDeviceToHost, st));
        collect_stats(G);
        check_device_error_public(env->ctx);
    });
}

int tn_ttn_env_product_flops(tn_ttn_env* env, double* flops) {
    return guarded([&] {
        TtnGroup& G = solo(env);
        TN_REQUIRE(flops, "null argument");
        *flops = product_plan(G, env->center).flops;
    });
}

int tn_ttn_env_set_projectors(tn_ttn_env* env, const tn_ttn* const* Ms, int count, double weight) {
    return guarded([&] {
        TN_REQUIRE(env && env->grp, "null argument");
        TN_REQUIRE(count >= 0 && count <= 32, "between 0 and 32 projector states");
        if (count > 0) {
            TN_REQUIRE(Ms, "null argument");
            if (!(weight > 0.0)) {
                char msg[160];
                std::snprintf(msg, sizeof msg,
                              "`weight` parameter should be > 0.0 (value passed was `weight=%g`)",
                              weight);
                throw Error(TN_E_INVALID, msg);
            }
            const TtnTree& t = env->tree;
            for (int k = 0; k < count; ++k) {
                const tn_ttn* M = Ms[k];
                TN_REQUIRE(M && M->ctx == env->ctx, "projector states must share the context");
                TN_REQUIRE(M->tree.N == t.N && M->tree.nn == t.nn && M->tree.d == t.d &&
                               M->tree.edges == t.edges && M->tree.site_node == t.site_node,
                           "projector states must have the tree and the sites of psi "
                           "(linkproj.jl:190-191)");
            }
        }
        proj_setup(*env->grp, env, Ms, count, weight);
        check_device_error_public(env->ctx);
    });
}

int tn_ttn_env_update_position(tn_ttn_env* env, int node, const tn_update_params* p,
                               tn_update_result* res) {
    return guarded([&] {
        TtnGroup& G = solo(env);
        TN_REQUIRE(node >= 0 && node < env->tree.nn, "bad node");
        update_group(G, node, p);
        collect_stats(G);
        check_device_error_public(env->ctx);
        if (res) {
            std::memset(res, 0, sizeof(*res));
            res->energy = env->energy;
            res->newdim = maxlinkdim_of(env->tree, env->dims);
            res->matvecs = env->matvecs;
            res->converged = env->converged;
        }
    });
}

int tn_ttn_envs_fullsweep_expand(int count, tn_ttn_env* const* envs, int npath,
                                 const int32_t* path, int central, const tn_update_params* p,
                                 int expand_dim, int max_expand_dim, int expand_numiter,
                                 uint64_t seed, tn_sweep_result* res) {
    return guarded([&] {
        TN_REQUIRE(count >= 1 && envs && envs[0] && path && res, "bad arguments");
        TtnGroup& G = *envs[0]->grp;
        TN_REQUIRE(count == G.alive && count == int(G.envs.size()),
                   "TTN: pass every environment of the group");
        for (int i = 0; i < count; ++i)
            TN_REQUIRE(envs[i] == G.envs[i], "TTN: environments must be given in creation order");
        const TtnTree& t = envs[0]->tree;
        std::vector<char> seen(t.nn, 0);
        for (int k = 0; k < npath; ++k) {
            TN_REQUIRE(path[k] >= 0 && path[k] < t.nn, "sweep path node out of range");
            seen[path[k]] = 1;
        }
        for (int v = 0; v < t.nn; ++v)
            TN_REQUIRE(seen[v], "the sweep path must contain every node (sweep_ttn.jl:120)");
        TN_REQUIRE(central >= 0 && central < t.nn, "central node out of range");
        check_ttn_params(p, true);
        TN_REQUIRE(p->noise > 0.0 && std::isfinite(p->noise), "noise must be > 0");
        TN_REQUIRE(expand_dim >= 0 && max_expand_dim >= 0, "expansion dimensions must be >= 0");
        if (expand_dim != 0 && expand_numiter < 2) {
            char msg[160];
            std::snprintf(msg, sizeof msg,
                          "`fullsweep!()`: `expand_numiter=%d` cannot be less than 2 for "
                          "`expand_dim=%d` !!", expand_numiter, expand_dim);
            throw Error(TN_E_INVALID, msg);
        }
        TN_REQUIRE(expand_numiter >= 1, "expand_numiter must be >= 1");
        reset_stats(G);
        const int64_t l0 = launch_count();
        const int64_t kb0 = krylov_bytes();
        const int s0 = G.ctx->timer.mark();
        fullsweep_expand(G, std::vector<int>(path, path + npath), p, central, expand_dim,
                         max_expand_dim, expand_numiter, seed);
        G.ctx->timer.add(T_SWEEP, s0, G.ctx->timer.mark());
        collect_stats(G);
        check_device_error_public(G.ctx);
        const int64_t launches = launch_count() - l0;
        G.krylov_bytes = double(krylov_bytes() - kb0);
        for (int i = 0; i < count; ++i) fill_sweep_result(G, envs[i], &res[i], launches);
    });
}

int tn_ttn_envs_fullsweep(int count, tn_ttn_env* const* envs, int npath, const int32_t* path,
                          const tn_update_params* p, tn_sweep_result* res) {
    return guarded([&] {
        TN_REQUIRE(count >= 1 && envs && envs[0] && path && res, "bad arguments");
        TtnGroup& G = *envs[0]->grp;
        TN_REQUIRE(count == G.alive && count == int(G.envs.size()),
                   "TTN: pass every environment of the group");
        for (int i = 0; i < count; ++i)
            TN_REQUIRE(envs[i] == G.envs[i], "TTN: environments must be given in creation order");
        const TtnTree& t = envs[0]->tree;
        std::vector<char> seen(t.nn, 0);
        for (int k = 0; k < npath; ++k) {
            TN_REQUIRE(path[k] >= 0 && path[k] < t.nn, "sweep path node out of range");
            seen[path[k]] = 1;
        }
        for (int v = 0; v < t.nn; ++v)
            TN_REQUIRE(seen[v], "the sweep path must contain every node (sweep_ttn.jl:120)");
        check_ttn_params(p);
        reset_stats(G);
        const int64_t l0 = launch_count();
        const int64_t kb0 = krylov_bytes();
        const int s0 = G.ctx->timer.mark();
        for (int k = 0; k < npath; ++k) update_group(G, path[k], p);
        for (int k = npath - 1; k >= 0; --k) update_group(G, path[k], p);
        G.ctx->timer.add(T_SWEEP, s0, G.ctx->timer.mark());
        collect_stats(G);
        check_device_error_public(G.ctx);
        const int64_t launches = launch_count() - l0;
        G.krylov_bytes = double(krylov_bytes() - kb0);
        for (int i = 0; i < count; ++i) fill_sweep_result(G, envs[i], &res[i], launches);
    });
}

}  // extern "C"
