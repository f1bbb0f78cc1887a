// Block layouts of U(1) charge-conserving tensors and the small host-side containers of
// contraction plans.
#include <algorithm>
#include <atomic>
#include <cstring>

#include "tn_internal.h"

namespace tn {

void cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    int code = (e == cudaErrorMemoryAllocation) ? -3 : -2;
    throw Error(code, std::string("CUDA error '") + cudaGetErrorString(e) + "' in " + what +
                          " at " + file + ":" + std::to_string(line));
}

static std::atomic<int64_t> g_launches{0};
int64_t launch_count() { return g_launches.load(); }
void count_launch(int n) { g_launches += n; }
static std::atomic<int64_t> g_krylov_bytes{0};
int64_t krylov_bytes() { return g_krylov_bytes.load(); }
void count_krylov_bytes(int64_t b) { g_krylov_bytes += b; }

void DevBuf::alloc(size_t nbytes, cudaStream_t s) {
    if (nbytes <= bytes && p) return;
    release();
    stream = s;
    if (nbytes == 0) nbytes = 16;
    nbytes = (nbytes + 255) & ~size_t(255);
    TN_CUDA(cudaMallocAsync(&p, nbytes, s));
    bytes = nbytes;
}

void DevBuf::release() {
    if (p) {
        cudaFreeAsync(p, stream);
        p = nullptr;
        bytes = 0;
    }
}

int Link::find(int charge) const {
    auto it = std::lower_bound(q.begin(), q.end(), charge);
    if (it == q.end() || *it != charge) return -1;
    return int(it - q.begin());
}
int Link::total() const {
    int t = 0;
    for (int x : dim) t += x;
    return t;
}
int Link::maxdim() const {
    int t = 0;
    for (int x : dim) t = std::max(t, x);
    return t;
}
std::vector<int> Link::offsets() const {
    std::vector<int> o(q.size());
    int t = 0;
    for (size_t i = 0; i < q.size(); ++i) {
        o[i] = t;
        t += dim[i];
    }
    return o;
}

SiteLayout make_site_layout(Layout lay, const Link& left, const Link& right,
                            const std::vector<int>& pq) {
    SiteLayout L;
    L.layout = lay;
    const int d = (int)pq.size();
    L.d = d;
    const Link& grp = (lay == LG) ? right : left;   // one block per sector of this link
    const Link& oth = (lay == LG) ? left : right;
    const int nb = grp.nsec();
    L.rows.resize(nb);
    L.cols.resize(nb);
    L.off.resize(nb);
    L.sub.assign(size_t(nb) * d, -1);
    L.subsec.assign(size_t(nb) * d, -1);
    int64_t off = 0;
    for (int b = 0; b < nb; ++b) {
        int acc = 0;
        for (int s = 0; s < d; ++s) {
            int other = (lay == LG) ? grp.q[b] - pq[s] : grp.q[b] + pq[s];
            int j = oth.find(other);
            if (j < 0) continue;
            L.sub[size_t(b) * d + s] = acc;
            L.subsec[size_t(b) * d + s] = j;
            acc += oth.dim[j];
        }
        if (lay == LG) {
            L.rows[b] = acc;
            L.cols[b] = grp.dim[b];
        } else {
            L.rows[b] = grp.dim[b];
            L.cols[b] = acc;
        }
        L.off[b] = off;
        off += int64_t(L.rows[b]) * L.cols[b];
    }
    L.size = off;
    return L;
}

int PhiLayout::find(int charge) const {
    auto it = std::lower_bound(m.begin(), m.end(), charge);
    if (it == m.end() || *it != charge) return -1;
    return int(it - m.begin());
}

PhiLayout make_phi_layout(const Link& left, const Link& right, const std::vector<int>& pq) {
    PhiLayout P;
    const int d = (int)pq.size();
    P.d = d;
    std::vector<int> cand;
    for (int l : left.q)
        for (int s = 0; s < d; ++s) cand.push_back(l + pq[s]);
    std::sort(cand.begin(), cand.end());
    cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
    int64_t off = 0;
    for (int mq : cand) {
        std::vector<int> rs(d, -1), rsec(d, -1), cs(d, -1), csec(d, -1);
        int nr = 0, nc = 0;
        for (int s = 0; s < d; ++s) {
            int j = left.find(mq - pq[s]);
            if (j >= 0) {
                rs[s] = nr;
                rsec[s] = j;
                nr += left.dim[j];
            }
        }
        for (int s = 0; s < d; ++s) {
            int j = right.find(mq + pq[s]);
            if (j >= 0) {
                cs[s] = nc;
                csec[s] = j;
                nc += right.dim[j];
            }
        }
        if (nr == 0 || nc == 0) continue;
        P.m.push_back(mq);
        P.rows.push_back(nr);
        P.cols.push_back(nc);
        P.off.push_back(off);
        off += int64_t(nr) * nc;
        P.rsub.insert(P.rsub.end(), rs.begin(), rs.end());
        P.rsec.insert(P.rsec.end(), rsec.begin(), rsec.end());
        P.csub.insert(P.csub.end(), cs.begin(), cs.end());
        P.csec.insert(P.csec.end(), csec.begin(), csec.end());
    }
    P.size = off;
    return P;
}

EnvLayout make_env_layout(const Link& link, const std::vector<int>& delta) {
    EnvLayout E;
    E.w = (int)delta.size();
    E.nsec = link.nsec();
    E.off.assign(size_t(E.w) * E.nsec, -1);
    E.bra.assign(size_t(E.w) * E.nsec, -1);
    int64_t off = 0;
    for (int a = 0; a < E.w; ++a)
        for (int x = 0; x < E.nsec; ++x) {
            int b = link.find(link.q[x] + delta[a]);
            if (b < 0) continue;
            E.off[size_t(a) * E.nsec + x] = off;
            E.bra[size_t(a) * E.nsec + x] = b;
            off += int64_t(link.dim[b]) * link.dim[x];
        }
    E.size = off;
    return E;
}

// ------------------------------------------------------------------------------------
// plan containers
// ------------------------------------------------------------------------------------
void GemmPlan::add_task(int cbuf, int64_t coff, int m, int n, int ldc, int accum) {
    Task t;
    t.accum = accum;
    t.coff = coff;
    t.cbuf = cbuf;
    t.m = m;
    t.n = n;
    t.ldc = ldc;
    t.seg0 = (int)segs.size();
    t.nseg = 0;
    tasks.push_back(t);
}

void GemmPlan::add_seg(int abuf, int64_t aoff, int lda, int ta, int bbuf, int64_t boff,
                       int ldb, int tb, int k, int sgn) {
    if (k <= 0) return;
    Seg s;
    s.sgn = sgn;
    s.aoff = aoff;
    s.boff = boff;
    s.abuf = abuf;
    s.bbuf = bbuf;
    s.lda = lda;
    s.ldb = ldb;
    s.k = k;
    s.ta = ta;
    s.tb = tb;
    segs.push_back(s);
    Task& t = tasks.back();
    t.nseg += 1;
    flops += 2.0 * double(t.m) * double(t.n) * double(k);
}

template <class T>
static void upload(DevBuf& b, const std::vector<T>& v, cudaStream_t s) {
    size_t nb = std::max<size_t>(v.size() * sizeof(T), 16);
    b.alloc(nb, s);
    if (!v.empty())
        TN_CUDA(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

void GemmPlan::finalize(cudaStream_t s) {
    tiles.clear();
    // heavy tasks first so that the tail of the grid is made of small tiles
    std::vector<int> order(tasks.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    auto work = [&](int i) {
        double k = 0;
        for (int j = 0; j < tasks[i].nseg; ++j) k += segs[tasks[i].seg0 + j].k;
        return k;
    };
    std::vector<double> w(tasks.size());
    for (size_t i = 0; i < tasks.size(); ++i) w[i] = work((int)i);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return w[a] > w[b]; });
    for (int ti : order) {
        const Task& t = tasks[ti];
        for (int m0 = 0; m0 < t.m; m0 += GEMM_BM)
            for (int n0 = 0; n0 < t.n; n0 += GEMM_BN) tiles.push_back(Tile{ti, m0, n0});
    }
    upload(dsegs, segs, s);
    upload(dtasks, tasks, s);
    upload(dtiles, tiles, s);
}

// (A_re + i a A_im)(B_re + i b B_im) = A_re B_re - a b A_im B_im + i (b A_re B_im + a A_im B_re)
// with a, b = -1 for a conjugated operand
GemmPlan complex_plan(const GemmPlan& g, unsigned conj_mask) {
    GemmPlan c;
    for (const Task& t : g.tasks) {
        for (int part = 0; part < 2; ++part) {
            c.add_task(t.cbuf + part * S_IM, t.coff, t.m, t.n, t.ldc, t.accum);
            for (int j = 0; j < t.nseg; ++j) {
                const Seg& s = g.segs[size_t(t.seg0 + j)];
                const int sa = (conj_mask >> s.abuf) & 1 ? -1 : 1;
                const int sb = (conj_mask >> s.bbuf) & 1 ? -1 : 1;
                const int ai = s.abuf + S_IM, bi = s.bbuf + S_IM;
                if (part == 0) {
                    c.add_seg(s.abuf, s.aoff, s.lda, s.ta, s.bbuf, s.boff, s.ldb, s.tb, s.k, s.sgn);
                    c.add_seg(ai, s.aoff, s.lda, s.ta, bi, s.boff, s.ldb, s.tb, s.k,
                              -sa * sb * s.sgn);
                } else {
                    c.add_seg(s.abuf, s.aoff, s.lda, s.ta, bi, s.boff, s.ldb, s.tb, s.k, sb * s.sgn);
                    c.add_seg(ai, s.aoff, s.lda, s.ta, s.bbuf, s.boff, s.ldb, s.tb, s.k, sa * s.sgn);
                }
            }
        }
    }
    return c;
}

CombPlan complex_comb(const CombPlan& c) {
    CombPlan z;
    z.outs = c.outs;
    z.terms = c.terms;
    z.flops = 2 * c.flops;
    const int nt = int(c.terms.size());
    for (CombTerm t : c.terms) {
        t.sbuf += S_IM;
        z.terms.push_back(t);
    }
    for (CombOut o : c.outs) {
        o.dbuf += S_IM;
        o.t0 += nt;
        z.outs.push_back(o);
    }
    return z;
}

void CombPlan::finalize(cudaStream_t s) {
    tiles.clear();
    for (size_t i = 0; i < outs.size(); ++i) {
        const CombOut& o = outs[i];
        for (int r0 = 0; r0 < o.rows; r0 += COMB_TR)
            for (int c0 = 0; c0 < o.cols; c0 += COMB_TC) tiles.push_back(CombTile{int(i), r0, c0});
    }
    upload(douts, outs, s);
    upload(dterms, terms, s);
    upload(dtiles, tiles, s);
}

}  // namespace tn
