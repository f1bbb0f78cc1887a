// Excited-state projectors of DMRG on the GPU: ProjMPS2 and ProjMPO_MPS2 (TenNetLib
// src/mps/projmps2.jl:26-224, src/mps/projmpo_mps2.jl:94-101).
//
// With states M_1..M_K held fixed the effective Hamiltonian becomes
// H_eff + w sum_k |m_k><m_k|, where m_k is M_k projected onto the sites being optimised:
// m_k = LM_k M_k[p] (M_k[p+1]) RM_k^T, with the overlap environments LM_k[i] (sites < i) and
// RM_k[i] (sites > i) of psi against M_k.  These are block-diagonal in the link charge
// (blocks D_psi(q) x D_M(q) for the charges both links carry).  They move with the MPO
// environments (two grouped FP64 GEMM launches per step), the m_k are formed once per
// position (two or three grouped GEMM launches), and each matvec adds the rank-K term with
// one dot launch (c = m^T x) and one axpy launch (y += w m c), all on the device.
#include <map>
#include <tuple>

#include "engine.h"

namespace tn {
namespace {

struct Sub {  // A_s[l, r] of one site: D_l x D_r at off (column-major, leading dim ld)
    int64_t off;
    int ld, l, r;  // sector indices of the left / right link
};
using SubMap = std::map<std::tuple<int, int, int>, Sub>;  // (s, left q, right q)

SubMap subs_of(const tn_mps* m, int i) {
    SubMap out;
    const SiteLayout& L = m->sites[i].lay;
    const int d = m->d;
    for (int b = 0; b < L.nblk(); ++b)
        for (int s = 0; s < d; ++s) {
            const int sub = L.sub[size_t(b) * d + s];
            if (sub < 0) continue;
            const int oth = L.subsec[size_t(b) * d + s];
            Sub x;
            x.ld = L.rows[b];
            if (L.layout == LG) {
                x.l = oth;
                x.r = b;
                x.off = L.off[b] + sub;
            } else {
                x.l = b;
                x.r = oth;
                x.off = L.off[b] + int64_t(sub) * L.rows[b];
            }
            if (m->links[i].dim[x.l] == 0 || m->links[i + 1].dim[x.r] == 0) continue;
            out[{s, m->links[i].q[x.l], m->links[i + 1].q[x.r]}] = x;
        }
    return out;
}

const Sub* find_sub(const SubMap& m, int s, int ql, int qr) {
    auto it = m.find({s, ql, qr});
    return it == m.end() ? nullptr : &it->second;
}

// blocks of the charges that both links carry, zeroed
void ov_layout(OvEnv& E, const Link& la, const Link& lb, cudaStream_t st) {
    E.q.clear();
    E.off.clear();
    E.da.clear();
    E.db.clear();
    int64_t tot = 0;
    for (int x = 0; x < la.nsec(); ++x) {
        const int y = lb.find(la.q[x]);
        if (y < 0 || la.dim[x] == 0 || lb.dim[y] == 0) continue;
        E.q.push_back(la.q[x]);
        E.da.push_back(la.dim[x]);
        E.db.push_back(lb.dim[y]);
        E.off.push_back(tot);
        tot += int64_t(la.dim[x]) * lb.dim[y];
    }
    E.size = tot;
    const size_t bytes = size_t(std::max<int64_t>(tot, 1)) * 8;
    E.buf.alloc(bytes, st);
    TN_CUDA(cudaMemsetAsync(E.buf.p, 0, bytes, st));
}

// LM[i+1] from LM[i]: E'(q_r) = sum_s A_s^T E(q_l) B_s  (ProjMPS2 _makeL!, projmps2.jl:76-91)
void ov_left(tn_ctx* ctx, const tn_mps* a, const tn_mps* b, int i, const OvEnv& Ein, OvEnv& Eout,
             DevBuf& tmp) {
    cudaStream_t st = ctx->stream;
    ov_layout(Eout, a->links[i + 1], b->links[i + 1], st);
    if (Ein.size == 0 || Eout.size == 0) return;
    const SubMap sa = subs_of(a, i), sb = subs_of(b, i);
    struct Job { const Sub *xa, *xb; int64_t toff; int ei, eo; };
    std::vector<Job> jobs;
    int64_t t = 0;
    for (const auto& kv : sa) {
        const Sub* xb = find_sub(sb, std::get<0>(kv.first), std::get<1>(kv.first),
                                 std::get<2>(kv.first));
        const int ei = Ein.find(std::get<1>(kv.first)), eo = Eout.find(std::get<2>(kv.first));
        if (!xb || ei < 0 || eo < 0) continue;
        jobs.push_back(Job{&kv.second, xb, t, ei, eo});
        t += int64_t(Ein.da[ei]) * Eout.db[eo];
    }
    if (jobs.empty()) return;
    tmp.alloc(size_t(t) * 8, st);
    GemmPlan g1, g2;
    std::map<int, std::vector<size_t>> byout;
    for (size_t k = 0; k < jobs.size(); ++k) {
        const Job& j = jobs[k];
        // T = E(q_l) (Da_l x Db_l) B_s (Db_l x Db_r)
        g1.add_task(S_T1, j.toff, Ein.da[j.ei], Eout.db[j.eo], Ein.da[j.ei]);
        g1.add_seg(S_L, Ein.off[j.ei], Ein.da[j.ei], 0, S_A, j.xb->off, j.xb->ld, 0, Ein.db[j.ei]);
        byout[j.eo].push_back(k);
    }
    for (const auto& kv : byout) {
        const int eo = kv.first;
        // E'(q_r) (Da_r x Db_r) = sum_s A_s^T T
        g2.add_task(S_R, Eout.off[eo], Eout.da[eo], Eout.db[eo], Eout.da[eo]);
        for (size_t k : kv.second) {
            const Job& j = jobs[k];
            g2.add_seg(S_X, j.xa->off, j.xa->ld, 1, S_T1, j.toff, Ein.da[j.ei], 0, Ein.da[j.ei]);
        }
    }
    g1.finalize(st);
    g2.finalize(st);
    Bases bs{};
    bs.p[S_L] = Ein.buf.d();
    bs.p[S_R] = Eout.buf.d();
    bs.p[S_X] = a->sites[i].buf.d();
    bs.p[S_A] = b->sites[i].buf.d();
    bs.p[S_T1] = tmp.d();
    launch_gemm_f64(g1, bs, st);
    launch_gemm_f64(g2, bs, st);
}

// RM[i-1] from RM[i]: E'(q_l) = sum_s A_s E(q_r) B_s^T  (ProjMPS2 _makeR!, projmps2.jl:106-122)
void ov_right(tn_ctx* ctx, const tn_mps* a, const tn_mps* b, int i, const OvEnv& Ein, OvEnv& Eout,
              DevBuf& tmp) {
    cudaStream_t st = ctx->stream;
    ov_layout(Eout, a->links[i], b->links[i], st);
    if (Ein.size == 0 || Eout.size == 0) return;
    const SubMap sa = subs_of(a, i), sb = subs_of(b, i);
    struct Job { const Sub *xa, *xb; int64_t toff; int ei, eo; };
    std::vector<Job> jobs;
    int64_t t = 0;
    for (const auto& kv : sa) {
        const Sub* xb = find_sub(sb, std::get<0>(kv.first), std::get<1>(kv.first),
                                 std::get<2>(kv.first));
        const int ei = Ein.find(std::get<2>(kv.first)), eo = Eout.find(std::get<1>(kv.first));
        if (!xb || ei < 0 || eo < 0) continue;
        jobs.push_back(Job{&kv.second, xb, t, ei, eo});
        t += int64_t(Eout.da[eo]) * Ein.db[ei];
    }
    if (jobs.empty()) return;
    tmp.alloc(size_t(t) * 8, st);
    GemmPlan g1, g2;
    std::map<int, std::vector<size_t>> byout;
    for (size_t k = 0; k < jobs.size(); ++k) {
        const Job& j = jobs[k];
        // T = A_s (Da_l x Da_r) E(q_r) (Da_r x Db_r)
        g1.add_task(S_T1, j.toff, Eout.da[j.eo], Ein.db[j.ei], Eout.da[j.eo]);
        g1.add_seg(S_X, j.xa->off, j.xa->ld, 0, S_L, Ein.off[j.ei], Ein.da[j.ei], 0, Ein.da[j.ei]);
        byout[j.eo].push_back(k);
    }
    for (const auto& kv : byout) {
        const int eo = kv.first;
        // E'(q_l) (Da_l x Db_l) = sum_s T B_s^T
        g2.add_task(S_R, Eout.off[eo], Eout.da[eo], Eout.db[eo], Eout.da[eo]);
        for (size_t k : kv.second) {
            const Job& j = jobs[k];
            g2.add_seg(S_T1, j.toff, Eout.da[eo], 0, S_A, j.xb->off, j.xb->ld, 1, Ein.db[j.ei]);
        }
    }
    g1.finalize(st);
    g2.finalize(st);
    Bases bs{};
    bs.p[S_L] = Ein.buf.d();
    bs.p[S_R] = Eout.buf.d();
    bs.p[S_X] = a->sites[i].buf.d();
    bs.p[S_A] = b->sites[i].buf.d();
    bs.p[S_T1] = tmp.d();
    launch_gemm_f64(g1, bs, st);
    launch_gemm_f64(g2, bs, st);
}

// the 1 x 1 edge block when the two states' edge charges agree (else empty: zero overlap)
void ov_edge(OvEnv& E, const Link& la, const Link& lb, cudaStream_t st) {
    ov_layout(E, la, lb, st);
    if (E.size == 1) {
        const double one = 1.0;
        TN_CUDA(cudaMemcpyAsync(E.buf.p, &one, 8, cudaMemcpyHostToDevice, st));
        TN_CUDA(cudaStreamSynchronize(st));  // the source is a stack value
    }
}

}  // namespace

int OvEnv::find(int charge) const {
    for (size_t x = 0; x < q.size(); ++x)
        if (q[x] == charge) return int(x);
    return -1;
}

void proj_init(tn_env* env) {
    const tn_mps* psi = env->psi.get();
    const int N = psi->N;
    cudaStream_t st = env->ctx->stream;
    for (ProjState& P : env->proj) {
        P.L.clear();
        P.R.clear();
        P.L.resize(N);
        P.R.resize(N);
        ov_edge(P.L[0], psi->links[0], P.M->links[0], st);
        ov_edge(P.R[N - 1], psi->links[N], P.M->links[N], st);
        for (int i = 0; i < env->lpos; ++i)
            ov_left(env->ctx, psi, P.M.get(), i, P.L[i], P.L[i + 1], env->projt1);
        for (int i = N - 1; i > env->rpos; --i)
            ov_right(env->ctx, psi, P.M.get(), i, P.R[i], P.R[i - 1], env->projt1);
    }
}

void proj_left_step(tn_env* env, int i) {
    for (ProjState& P : env->proj)
        ov_left(env->ctx, env->psi.get(), P.M.get(), i, P.L[i], P.L[i + 1], env->projt1);
}

void proj_right_step(tn_env* env, int i) {
    for (ProjState& P : env->proj)
        ov_right(env->ctx, env->psi.get(), P.M.get(), i, P.R[i], P.R[i - 1], env->projt1);
}

// proj_mps (projmps2.jl:168-184) of every M_k at the bond (p, p+1), in the two-site layout:
// m[l, s1, s2, r] = sum LM(l, a) M_p[a, s1, x] M_p+1[x, s2, b] RM(r, b)
void proj_vectors2(tn_env* env, int p, const PhiLayout& ph) {
    const tn_mps* psi = env->psi.get();
    tn_ctx* ctx = env->ctx;
    cudaStream_t st = ctx->stream;
    const int K = int(env->proj.size()), d = psi->d;
    const int64_t n = ph.size;
    const size_t bytes = size_t(std::max<int64_t>(int64_t(K) * n, 1)) * 8;
    env->projm.alloc(bytes, st);
    TN_CUDA(cudaMemsetAsync(env->projm.p, 0, bytes, st));
    const Link& lk = psi->links[p];
    const Link& rk = psi->links[p + 2];
    for (int k = 0; k < K; ++k) {
        const ProjState& P = env->proj[k];
        const tn_mps* M = P.M.get();
        const OvEnv& LM = P.L[p];
        const OvEnv& RM = P.R[p + 1];
        if (LM.size == 0 || RM.size == 0) continue;
        const SubMap s0 = subs_of(M, p), s1m = subs_of(M, p + 1);
        GemmPlan g1, g2, g3;
        int64_t t1 = 0, t2 = 0;
        for (int mi = 0; mi < ph.nblk(); ++mi) {
            const int qm = ph.m[mi];
            const int xm = M->links[p + 1].find(qm);
            if (xm < 0 || M->links[p + 1].dim[xm] == 0) continue;
            const int Dx = M->links[p + 1].dim[xm];
            for (int s1 = 0; s1 < d; ++s1) {
                const int rs = ph.rsub[size_t(mi) * d + s1];
                if (rs < 0) continue;
                const int il = ph.rsec[size_t(mi) * d + s1];
                const int el = LM.find(lk.q[il]);
                const Sub* a = find_sub(s0, s1, lk.q[il], qm);
                if (el < 0 || !a) continue;
                const int Dl = LM.da[el];
                const int64_t o1 = t1;
                // T1 = LM(q_l) (Dl x DM_l) M_p[s1] (DM_l x Dx)
                g1.add_task(S_T1, o1, Dl, Dx, Dl);
                g1.add_seg(S_L, LM.off[el], Dl, 0, S_A, a->off, a->ld, 0, LM.db[el]);
                t1 += int64_t(Dl) * Dx;
                for (int s2 = 0; s2 < d; ++s2) {
                    const int cs = ph.csub[size_t(mi) * d + s2];
                    if (cs < 0) continue;
                    const int ir = ph.csec[size_t(mi) * d + s2];
                    const int er = RM.find(rk.q[ir]);
                    const Sub* b = find_sub(s1m, s2, qm, rk.q[ir]);
                    if (er < 0 || !b) continue;
                    const int DMr = RM.db[er], Dr = RM.da[er];
                    // T2 = T1 (Dl x Dx) M_p+1[s2] (Dx x DM_r)
                    g2.add_task(S_T2, t2, Dl, DMr, Dl);
                    g2.add_seg(S_T1, o1, Dl, 0, S_B, b->off, b->ld, 0, Dx);
                    // m block (Dl x Dr) = T2 RM(q_r)^T
                    g3.add_task(S_Y, int64_t(k) * n + ph.off[mi] + rs + int64_t(cs) * ph.rows[mi],
                                Dl, Dr, ph.rows[mi]);
                    g3.add_seg(S_T2, t2, Dl, 0, S_R, RM.off[er], Dr, 1, DMr);
                    t2 += int64_t(Dl) * DMr;
                }
            }
        }
        if (g3.tasks.empty()) continue;
        env->projt1.alloc(size_t(std::max<int64_t>(t1, 1)) * 8, st);
        env->projt2.alloc(size_t(std::max<int64_t>(t2, 1)) * 8, st);
        g1.finalize(st);
        g2.finalize(st);
        g3.finalize(st);
        Bases bs{};
        bs.p[S_L] = LM.buf.d();
        bs.p[S_R] = RM.buf.d();
        bs.p[S_A] = M->sites[p].buf.d();
        bs.p[S_B] = M->sites[p + 1].buf.d();
        bs.p[S_T1] = env->projt1.d();
        bs.p[S_T2] = env->projt2.d();
        bs.p[S_Y] = env->projm.d();
        launch_gemm_f64(g1, bs, st);
        launch_gemm_f64(g2, bs, st);
        launch_gemm_f64(g3, bs, st);
    }
}

// the same at site p in the right-grouped one-site layout: m = LM M_p RM^T
void proj_vectors1(tn_env* env, int p, const SiteLayout& lay) {
    const tn_mps* psi = env->psi.get();
    cudaStream_t st = env->ctx->stream;
    const int K = int(env->proj.size()), d = psi->d;
    const int64_t n = lay.size;
    const size_t bytes = size_t(std::max<int64_t>(int64_t(K) * n, 1)) * 8;
    env->projm.alloc(bytes, st);
    TN_CUDA(cudaMemsetAsync(env->projm.p, 0, bytes, st));
    TN_REQUIRE(lay.layout == RG, "internal: one-site projector layout");
    const Link& lk = psi->links[p];
    const Link& rk = psi->links[p + 1];
    for (int k = 0; k < K; ++k) {
        const ProjState& P = env->proj[k];
        const tn_mps* M = P.M.get();
        const OvEnv& LM = P.L[p];
        const OvEnv& RM = P.R[p];
        if (LM.size == 0 || RM.size == 0) continue;
        const SubMap s0 = subs_of(M, p);
        GemmPlan g1, g3;
        int64_t t1 = 0;
        for (int b = 0; b < lay.nblk(); ++b) {
            const int el = LM.find(lk.q[b]);
            if (el < 0) continue;
            const int Dl = LM.da[el];
            for (int s = 0; s < d; ++s) {
                const int sub = lay.sub[size_t(b) * d + s];
                if (sub < 0) continue;
                const int ir = lay.subsec[size_t(b) * d + s];
                const int er = RM.find(rk.q[ir]);
                const Sub* a = find_sub(s0, s, lk.q[b], rk.q[ir]);
                if (er < 0 || !a) continue;
                const int DMr = RM.db[er], Dr = RM.da[er];
                // T1 = LM(q_l) (Dl x DM_l) M_p[s] (DM_l x DM_r); m block = T1 RM(q_r)^T
                g1.add_task(S_T1, t1, Dl, DMr, Dl);
                g1.add_seg(S_L, LM.off[el], Dl, 0, S_A, a->off, a->ld, 0, LM.db[el]);
                g3.add_task(S_Y, int64_t(k) * n + lay.off[b] + int64_t(sub) * lay.rows[b], Dl, Dr,
                            lay.rows[b]);
                g3.add_seg(S_T1, t1, Dl, 0, S_R, RM.off[er], Dr, 1, DMr);
                t1 += int64_t(Dl) * DMr;
            }
        }
        if (g3.tasks.empty()) continue;
        env->projt1.alloc(size_t(std::max<int64_t>(t1, 1)) * 8, st);
        g1.finalize(st);
        g3.finalize(st);
        Bases bs{};
        bs.p[S_L] = LM.buf.d();
        bs.p[S_R] = RM.buf.d();
        bs.p[S_A] = M->sites[p].buf.d();
        bs.p[S_T1] = env->projt1.d();
        bs.p[S_Y] = env->projm.d();
        launch_gemm_f64(g1, bs, st);
        launch_gemm_f64(g3, bs, st);
    }
}

// y += w sum_k m_k (m_k . x)  (ProjMPO_MPS2 product, projmpo_mps2.jl:94-101)
void proj_apply(tn_env* env, const double* x, double* y, int64_t n) {
    const int K = int(env->proj.size());
    if (K == 0) return;
    cudaStream_t st = env->ctx->stream;
    std::vector<const double*> m(K);
    for (int k = 0; k < K; ++k) m[k] = env->projm.d() + int64_t(k) * n;
    env->projc.alloc(64 * 8, st);
    launch_multi_dot(m.data(), K, x, n, env->part.d(), env->projc.d(), st);
    launch_multi_axpy(y, m.data(), K, env->projc.d(), env->proj_weight, n, st);
}

}  // namespace tn
